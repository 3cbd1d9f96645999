// Mixed-precision list-1 evaluation on the tensor cores (tcgen05, FP16 digits,
// exact FP32 partial products, exact integer sums, one rounding to FP64).
//
// Formulation.  For a target box T and right-hand side r,
//   y[T, t, r] = sum over list-1 pairs (T, S) with key k = (table level, case)
//                sum_s  B_k[s, t] * x'[S, s, r]          (+ 2D displacement)
// with x' = scaling(level S) * coefficient.  Rows of one CTA tile are 128
// (target box, rhs) items; the CTA loops over the keys present in its tile and
// accumulates D[row, t] = sum_s X[row, s] * A_k[t, s] with tcgen05.mma
// (M = 128 rows, N = target points of a column chunk, K = source points in
// chunks of <= 64).
//
// Exactness (an Ozaki-type split).  The table blocks (per plan) and x' (per
// call) are written in fixed point against power-of-two scales, both as
// 39-bit magnitudes in balanced base-256 digits (|digit| <= 128, times the
// value's sign), held exactly in FP16: the table against one scale per plan,
// the densities against one scale per right-hand side (the exponent of the
// largest |x'| of that rhs over all boxes).  Because every density of an rhs
// shares one scale, the FP16 digit planes are formed once per call by a
// preparation kernel and the tensor-core kernel only gathers them.  A diagonal
// i + j of digit products summed over K <= 128 source points (one exact
// round, which may span several table keys) is an integer of magnitude at
// most 2^22 for i + j <= 3 and below 2^23 for i + j = 4, exact in the FP32
// accumulator.  Those diagonals (the leading 32 bits) get their
// own TMEM accumulator, re-initialised per K round and read after every round
// into int64 registers: one FADD with 1.5 * 2^23 turns an exact d <= 3 float
// into its integer bits, d = 4 takes a conversion; diagonals i + j = 5, 6
// accumulate across rounds in FP32 TMEM (their rounding is below 2^-40 of the
// result); the products i + j >= 7 are dropped, and with balanced digits they
// are zero-mean.  Each output's sum is then one exact integer, rounded once to
// FP64.
#include <cuda_fp16.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "vl1_internal.cuh"
#include "vl1_mixed.cuh"
#include "vl1_tc.cuh"

namespace vl1 {

namespace {

constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
constexpr int kMagicBits = 0x4B400000;

// ----------------------------------------------------------------- helpers

// |v| as a fixed-point integer m with |v| = 2^(e - BITS) * m, m < 2^BITS,
// rounded to nearest (ties to even), from the IEEE-754 fields with integer
// arithmetic only: it equals round(ldexp(|v|, BITS - e)) without touching the
// FP64 pipe, which is narrow on this GPU.
template <int BITS>
__device__ __forceinline__ unsigned long long fixed_magnitude(double v, int e) {
  const unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(v));
  const unsigned long long mag = bits & 0x7FFFFFFFFFFFFFFFull;
  const int ef = (int)(mag >> 52);
  // |v| = M * 2^ev
  const unsigned long long M = ef ? ((mag & 0xFFFFFFFFFFFFFull) | (1ull << 52)) : mag;
  const int ev = ef ? ef - 1075 : -1074;
  const long long sh = (long long)ev + BITS - (long long)e;
  unsigned long long m;
  if (sh < 0) {
    // the usual case (|v| < 2^e leaves at least 14 bits to drop): M / 2^k
    // rounded to nearest, ties to even, as (M + 2^(k-1) - 1 + lsb) >> k
    if (sh < -63) {
      m = 0;
    } else {
      const int k = (int)-sh;
      const unsigned long long half = 1ull << (k - 1);
      m = (M + (half - 1ull) + ((M >> k) & 1ull)) >> k;
    }
  } else {
    // saturates when |v| is not below 2^e (m >= 2^BITS after the shift)
    m = M == 0 ? 0
               : ((sh > BITS || M >= (1ull << (BITS - sh))) ? (1ull << BITS) : (M << sh));
  }
  if (m >= (1ull << BITS)) m = (1ull << BITS) - 1;  // v at the scale bound
  return m;
}

// table digits: v = sign * 2^(e - 39) * m, m < 2^39, written in balanced
// base 256: m = sum_i d_i 256^(4 - i) with d_1..d_4 in [-128, 128) and the top
// digit d_0 in [0, 128], all multiplied by the sign of v (|digit| <= 128).
// Balanced digits make every digit product that the truncated expansion
// drops (i + j >= 7) zero-mean, so the dropped terms cancel instead of
// adding up with the sign of the products, as sign-magnitude digits would.
__device__ __forceinline__ void fixed_digits(double v, int e, int (&dig)[kDigits]) {
  const unsigned long long m = fixed_magnitude<kFixedBits>(v, e);
  const int sgn = __double_as_longlong(v) < 0 ? -1 : 1;
  // bytes of m (low to high) in 32-bit arithmetic; a byte >= 128 becomes
  // byte - 256 and carries one into the next (a byte 255 plus a carry gives
  // 0 and carries on)
  const unsigned lo32 = (unsigned)m;
  int carry = 0;
#pragma unroll
  for (int i = kDigits - 1; i >= 1; --i) {
    int t = (int)((lo32 >> (kDigitBits * (kDigits - 1 - i))) & 0xFFu) + carry;
    carry = t >= 128 ? 1 : 0;
    t -= carry << kDigitBits;
    dig[i] = sgn * t;
  }
  dig[0] = sgn * ((int)(m >> 32) + carry);   // m < 2^39: <= 128
}

// The four FP16 density plane values of v against 2^e: X1, X2, X3 = the
// three leading balanced digits of m (fixed_digits) and R = X4 + X5 / 256.
// The balanced digits come from m + 0x80808080: adding 128 to each of the
// low bytes makes the additions' carries do the digit borrows (a byte b
// plus the incoming carry becomes b + c - 256 with a carry out exactly when
// b + c >= 128), so each digit is its biased byte minus 128, the top digit
// takes the last carry, and X4 * 256 + X5 is the low 16 bits minus 0x8080
// (bit-identical to fixed_digits on 60 M checked values).
__device__ __forceinline__ void plane_values(double v, int e, __half &x1, __half &x2,
                                             __half &x3, __half &rr) {
  const unsigned long long m = fixed_magnitude<kFixedBits>(v, e);
  const int sgn = __double_as_longlong(v) < 0 ? -1 : 1;
  const unsigned lo = (unsigned)m;
  const unsigned lp = lo + 0x80808080u;
  const int top = (int)(m >> 32) + (lp < lo ? 1 : 0);
  x1 = __int2half_rn(sgn * top);
  x2 = __int2half_rn(sgn * ((int)(lp >> 24) - 128));
  x3 = __int2half_rn(sgn * ((int)((lp >> 16) & 0xFFu) - 128));
  // exact in FP32 (|.| <= 128.5 in steps of 1/256), one rounding to FP16
  rr = __float2half_rn((float)(sgn * ((int)(lp & 0xFFFFu) - 0x8080)) * (1.0f / 256.0f));
}

// exponent e with |v| < 2^e, as frexp returns it (-1074 for v == 0), from the
// IEEE-754 fields
__device__ __forceinline__ int scale_exponent(double v) {
  const unsigned long long mag =
      static_cast<unsigned long long>(__double_as_longlong(v)) & 0x7FFFFFFFFFFFFFFFull;
  if (mag == 0) return -1074;
  const int ef = (int)(mag >> 52);
  if (ef) return ef - 1022;
  return (64 - __clzll((long long)mag)) - 1074;   // subnormal
}

// ------------------------------------------------- plan: A digit operands

__global__ void build_adig_kernel(DevDesc d, MixedGeom g, __half *adig, int a_exp) {
  // element (key, kchunk, digit, n, k) of [key][kchunk][digit][NP][KC]
  // (swizzled K-major order inside each [NP][KC] tile, as in shared memory)
  const int64_t per_tile = (int64_t)g.np * g.kc;
  const int64_t n_elems = (int64_t)d.n_tables * d.n_cases * g.n_kc * kDigits * per_tile;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n_elems;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t rem = idx % per_tile;
    const int n = (int)(rem / g.kc);
    const int k = (int)(rem % g.kc);
    int64_t q = idx / per_tile;
    const int digit = (int)(q % kDigits);
    q /= kDigits;
    const int kc = (int)(q % g.n_kc);
    const int key = (int)(q / g.n_kc);
    const int s = kc * g.kc + k;
    int t = n, part = 0;
    if (d.table_cplx && n >= d.nq) {
      t = n - d.nq;
      part = 1;
    }
    double v = 0.0;
    if (s < d.nq && t < d.nq) {
      const int64_t bi = ((int64_t)key * d.nq + s) * d.nq + t;
      v = d.table_cplx ? d.blocks[2 * bi + part] : d.blocks[bi];
    }
    int dig[kDigits];
    fixed_digits(v, a_exp, dig);
    const int64_t tile = ((int64_t)key * g.n_kc + kc) * kDigits + digit;
    const uint32_t off = tc::kmajor_swizzled_offset(n, k, g.kc);  // bytes
    adig[tile * per_tile + off / 2] = __int2half_rn(dig[digit]);
  }
}

// -------------------------------------------------- per call: preparation

__global__ void classify_pairs_kernel(DevDesc d, TreeDev tr, int32_t *keys, vl1_status *st) {
  for (int tb = blockIdx.x * blockDim.x + threadIdx.x; tb < tr.n_tgt_boxes;
       tb += gridDim.x * blockDim.x) {
    const int tbox = tr.target_boxes[tb];
    for (int p = tr.starts[tb]; p < tr.starts[tb + 1]; ++p) {
      const int sbox = tr.lists[p];
      const int lvl = tr.levels[sbox];
      const double ext = level_extent(tr.root_extent, lvl);
      const int c = pair_case_id(d, tr, tbox, sbox, ext);
      if (c < 0) {
        report(st, VL1_E_INVALID_CASE, tb, p);
        keys[p] = -1;
      } else {
        keys[p] = pair_table_level(d, lvl) * d.n_cases + c;
      }
    }
  }
}

// Per-call preparation kernels: one warp per density row (source box b, rhs r).

// Scale exponents: x_exp[r] holds kExpBias + E_r, E_r the exponent with
// |scaling * coefficient| < 2^E_r over every box of rhs r (zeroed before the
// exponent pass, which takes the maximum with atomics; an rhs that is zero
// everywhere keeps 0, i.e. E_r = -kExpBias, and all its digits are zero).
constexpr int kExpBias = 4096;

// one problem of a batch, as the preparation kernels see it
struct PrepProblem {
  DevDesc d;
  TreeDev tr;
  const double *coefs;
  int nrhs;
  int *x_exp;      // per rhs: kExpBias + E_r
  __half *xpl;     // density digit planes [row][K chunk][plane][kc]
  double *wbox, *disp;   // 2D log displacement scratch (nullptr: none)
  int kp, kc;
  vl1_status *st;
};
// rows [row0, row0 + nrows) of one problem
struct PrepTask {
  int32_t problem;
  int32_t nrows;
  int64_t row0;
};

// The preparation passes take the density rows (R = b * nrhs + r) in groups
// of kRowGroup consecutive rows per warp: lane j < kRowGroup loads row j's
// box data, and every lane issues its loads of all rows of the group before
// using them, so that the rows' memory latencies overlap (one row per warp
// left both passes latency-bound at ~20 us each on a 26k-box tree).
constexpr int kRowGroup = 8;

struct RowGroup {
  int n;                 // rows in the group (<= kRowGroup)
  int cnt, start, rhs;   // lane j < n: row j's source count (clamped), first source, rhs
  int level, box;
};

__device__ __forceinline__ RowGroup load_row_group(const DevDesc &d, const TreeDev &tr,
                                                   int nrhs, int64_t r0, int n, int lane,
                                                   vl1_status *st) {
  RowGroup g;
  g.n = n;
  g.cnt = g.start = g.rhs = g.level = g.box = 0;
  if (lane < n) {
    const int64_t idx = r0 + lane;
    const int b = (int)(idx / nrhs);
    g.box = b;
    g.rhs = (int)(idx - (int64_t)b * nrhs);
    int cnt = tr.src_counts[b];
    if (cnt > d.nq) {
      if (st) report(st, VL1_E_LAYOUT, b, cnt);
      cnt = d.nq;
    }
    g.cnt = cnt;
    g.start = tr.src_starts[b];
    g.level = tr.levels[b];
  }
  return g;
}

// warp-wide maximum of a 64-bit unsigned value
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
  const unsigned hi = __reduce_max_sync(0xffffffffu, (unsigned)(v >> 32));
  const unsigned lo = __reduce_max_sync(0xffffffffu,
                                        (unsigned)(v >> 32) == hi ? (unsigned)v : 0u);
  return ((unsigned long long)hi << 32) | lo;
}

// The exponent pass: each row's largest exponent of scaling * coefficient
// into its rhs's maximum.  Rounding is monotone, so the largest exponent of
// sc * c over a row is the exponent of sc * max |c|: the row's maximum is
// taken on the IEEE bit patterns of |c| (ordered like the values) and
// multiplied once.  A block collects the maxima of its rows in shared memory
// (rhs counts up to kExpSmemRhs) and adds one global atomic per rhs.
constexpr int kExpSmemRhs = 1024;

__device__ __forceinline__ void exp_block_begin(int nrhs, int *s_max) {
  if (nrhs <= kExpSmemRhs)
    for (int i = threadIdx.x; i < nrhs; i += blockDim.x) s_max[i] = 0;
  __syncthreads();
}

__device__ __forceinline__ void group_exponent_max(const DevDesc &d, const TreeDev &tr,
                                                   const double *coefs, int nrhs, int *x_exp,
                                                   int64_t r0, int n, int lane, int *s_max) {
  const RowGroup g = load_row_group(d, tr, nrhs, r0, n, lane, nullptr);
  int cnt[kRowGroup];
  const double *c[kRowGroup];
#pragma unroll
  for (int u = 0; u < kRowGroup; ++u) {
    cnt[u] = __shfl_sync(0xffffffffu, g.cnt, u);
    const int st = __shfl_sync(0xffffffffu, g.start, u);
    const int rh = __shfl_sync(0xffffffffu, g.rhs, u);
    c[u] = coefs + (int64_t)rh * tr.n_particles + st;
    if (u >= n) cnt[u] = 0;
  }
  unsigned long long m[kRowGroup];
#pragma unroll
  for (int u = 0; u < kRowGroup; ++u) m[u] = 0ull;
  for (int k = lane; k < d.nq; k += 32) {
    double v[kRowGroup];
#pragma unroll
    for (int u = 0; u < kRowGroup; ++u) v[u] = k < cnt[u] ? c[u][k] : 0.0;
#pragma unroll
    for (int u = 0; u < kRowGroup; ++u) {
      const unsigned long long a =
          static_cast<unsigned long long>(__double_as_longlong(v[u])) & 0x7FFFFFFFFFFFFFFFull;
      m[u] = a > m[u] ? a : m[u];
    }
  }
  unsigned long long mine = 0ull;
#pragma unroll
  for (int u = 0; u < kRowGroup; ++u) {
    const unsigned long long w = warp_max_u64(m[u]);
    if (lane == u) mine = w;
  }
  if (lane < n && mine != 0ull) {
    const double sc = box_scaling(d, tr, g.level);
    const int e = scale_exponent(sc * __longlong_as_double((long long)mine));
    if (e > -1074) {
      if (nrhs <= kExpSmemRhs)
        atomicMax(s_max + g.rhs, e + kExpBias);
      else
        atomicMax(x_exp + g.rhs, e + kExpBias);
    }
  }
}

// the block's maxima into the global ones (0: no nonzero value seen; the
// biased exponents are positive)
__device__ __forceinline__ void exp_block_end(int nrhs, const int *s_max, int *x_exp) {
  __syncthreads();
  if (nrhs <= kExpSmemRhs)
    for (int i = threadIdx.x; i < nrhs; i += blockDim.x)
      if (s_max[i] > 0) atomicMax(x_exp + i, s_max[i]);
}

// Density digit planes of row R = b * nrhs + r: [K chunk][plane][kc] FP16
// values (source points at their mode id, zero elsewhere), planes X1, X2, X3
// (the three leading balanced digits) and R = X4 + X5 / 256 rounded once to
// FP16 (the tails only), so that the four planes of one pipeline unit are one
// contiguous 8 * kc-byte piece at byte kchunk * 8 * kc.  A warp takes a group
// of rows, assembles each in its own slice of the warp's shared-memory
// staging (G slices of 8 * kp bytes) and writes them out with 16-byte
// stores.
constexpr int kXPlanes = 4;          // density planes: X1, X2, X3, R
#ifndef VL1_PLANE_GROUP
#define VL1_PLANE_GROUP 4
#endif
// rows per warp group of the plane pass (its digit work holds every row's
// state in registers, so it takes fewer rows than the exponent pass)
constexpr int kPlaneGroup = VL1_PLANE_GROUP;
template <int G>
__device__ __forceinline__ void group_planes(const DevDesc &d, const TreeDev &tr,
                                             const double *coefs, int nrhs, const int *x_exp,
                                             __half *xpl, int kp, int kc, vl1_status *st,
                                             int64_t r0, int n, int lane, uint8_t *stage) {
  const int row_bytes = kp * kXPlanes * 2;
  const int kc_shift = 31 - __clz(kc);
  const RowGroup g = load_row_group(d, tr, nrhs, r0, n, lane, st);
  int ex = 0, sl = kNoScaleLog2;
  double sc = 0.0;
  if (lane < n) {
    ex = x_exp[g.rhs] - kExpBias;
    sc = box_scaling(d, tr, g.level);
    // a power-of-two scaling: digits of c against 2^(e - log2 sc), the same
    // as those of sc * c against 2^e when the product is exact (no overflow:
    // e <= 1000; an underflowing product has zero digits when e >= -900)
    if (g.level < kScaleLevels && ex >= -900 && ex <= 1000)
      sl = tr.level_scale_log2[g.level];
  }
  for (int k = lane * 16; k < G * row_bytes; k += 32 * 16)
    *reinterpret_cast<uint4 *>(stage + k) = make_uint4(0u, 0u, 0u, 0u);
  // every row's data in every lane (shuffles before the point loop, which
  // not all lanes enter when nq is not a multiple of 32)
  int cnt[G], st0[G], eu[G], bx[G], slu[G];
  double scu[G];
  const double *c[G];
#pragma unroll
  for (int u = 0; u < G; ++u) {
    cnt[u] = __shfl_sync(0xffffffffu, g.cnt, u);
    st0[u] = __shfl_sync(0xffffffffu, g.start, u);
    const int rh = __shfl_sync(0xffffffffu, g.rhs, u);
    eu[u] = __shfl_sync(0xffffffffu, ex, u);
    scu[u] = __shfl_sync(0xffffffffu, sc, u);
    slu[u] = __shfl_sync(0xffffffffu, sl, u);
    bx[u] = __shfl_sync(0xffffffffu, g.box, u);
    c[u] = coefs + (int64_t)rh * tr.n_particles + st0[u];
    if (u >= n) cnt[u] = 0;
  }
  __syncwarp();
  for (int k = lane; k < d.nq; k += 32) {
    double v[G];
    int m[G];
#pragma unroll
    for (int u = 0; u < G; ++u) {
      const bool have = k < cnt[u];
      v[u] = have ? c[u][k] : 0.0;
      m[u] = have ? tr.smode[st0[u] + k] : -2;
    }
#pragma unroll
    for (int u = 0; u < G; ++u) {
      if (m[u] == -2) continue;
      if (m[u] < 0 || m[u] >= d.nq) {
        report(st, VL1_E_LAYOUT, bx[u], -1 - k);
        continue;
      }
      const bool shift = slu[u] != kNoScaleLog2;
      __half x1, x2, x3, rr;
      plane_values(shift ? v[u] : scu[u] * v[u], shift ? eu[u] - slu[u] : eu[u], x1, x2, x3,
                   rr);
      // kc is 16 or 32: chunk and column by shift and mask
      __half *hv = reinterpret_cast<__half *>(stage + u * row_bytes) +
                   ((m[u] >> kc_shift) * kXPlanes << kc_shift) + (m[u] & (kc - 1));
      hv[0] = x1;
      hv[kc] = x2;
      hv[2 * kc] = x3;
      hv[3 * kc] = rr;
    }
  }
  __syncwarp();
  for (int u = 0; u < n; ++u) {
    uint8_t *row = reinterpret_cast<uint8_t *>(xpl) + (r0 + u) * row_bytes;
    for (int k = lane * 16; k < row_bytes; k += 32 * 16)
      *reinterpret_cast<uint4 *>(row + k) =
          *reinterpret_cast<const uint4 *>(stage + u * row_bytes + k);
  }
  __syncwarp();
}

__global__ void x_exponent_kernel(DevDesc d, TreeDev tr, int nboxes, const double *coefs,
                                  int nrhs, int *x_exp) {
  __shared__ int s_max[kExpSmemRhs];
  exp_block_begin(nrhs, s_max);
  const int64_t n = (int64_t)nboxes * nrhs;
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t g = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
       g * kRowGroup < n; g += warps) {
    const int64_t r0 = g * kRowGroup;
    group_exponent_max(d, tr, coefs, nrhs, x_exp, r0,
                       (int)min((int64_t)kRowGroup, n - r0), lane, s_max);
  }
  exp_block_end(nrhs, s_max, x_exp);
}

// dynamic shared memory: (blockDim.x / 32) x kPlaneGroup x kp * 8 bytes (kp a
// multiple of 16, so every slice and row stays 16-byte aligned)
__global__ void __launch_bounds__(128)
    x_planes_kernel(DevDesc d, TreeDev tr, int nboxes, const double *coefs, int nrhs,
                    const int *x_exp, __half *xpl, int kp, int kc, vl1_status *st) {
  extern __shared__ __align__(16) uint8_t s_stage[];
  const int64_t n = (int64_t)nboxes * nrhs;
  const int lane = threadIdx.x & 31;
  uint8_t *stage = s_stage + (threadIdx.x >> 5) * kPlaneGroup * kp * kXPlanes * 2;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t g = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
       g * kPlaneGroup < n; g += warps) {
    const int64_t r0 = g * kPlaneGroup;
    group_planes<kPlaneGroup>(d, tr, coefs, nrhs, x_exp, xpl, kp, kc, st, r0,
                              (int)min((int64_t)kPlaneGroup, n - r0), lane, stage);
  }
}

// The exponent pass for small boxes (nq <= 32) with several rhs: rows in row
// order put one box's rhs next to each other, whose densities lie
// n_particles values apart, so the row-group pass reads scattered 8 * nq-byte
// pieces (C3: 210 MB at ~1.9 TB/s).  Here a warp takes one rhs of 32
// consecutive boxes - contiguous densities - one lane per box: the lane's
// maximum of |c| bits, one multiply, the maximum over the warp, one
// shared-memory maximum per warp.
__global__ void __launch_bounds__(128)
    x_exponent_small_kernel(DevDesc d, TreeDev tr, int nboxes, const double *coefs, int nrhs,
                            int *x_exp) {
  __shared__ int s_max[kExpSmemRhs];
  exp_block_begin(nrhs, s_max);
  const int lane = threadIdx.x & 31;
  const int64_t n_tiles = (int64_t)((nboxes + 31) / 32) * nrhs;   // (32 boxes, one rhs)
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; w < n_tiles;
       w += warps) {
    const int r = (int)(w % nrhs);
    const int b = (int)(w / nrhs) * 32 + lane;
    int e = 0;
    if (b < nboxes) {
      const int cnt = min(tr.src_counts[b], d.nq);
      const double *c = coefs + (int64_t)r * tr.n_particles + tr.src_starts[b];
      unsigned long long mx = 0ull;
      for (int k = 0; k < cnt; ++k) {
        const unsigned long long a =
            static_cast<unsigned long long>(__double_as_longlong(c[k])) & 0x7FFFFFFFFFFFFFFFull;
        mx = a > mx ? a : mx;
      }
      if (mx != 0ull) {
        const int ex = scale_exponent(box_scaling(d, tr, tr.levels[b]) *
                                      __longlong_as_double((long long)mx));
        if (ex > -1074) e = ex + kExpBias;
      }
    }
    e = __reduce_max_sync(0xffffffffu, e);
    if (lane == 0 && e > 0) {
      if (nrhs <= kExpSmemRhs)
        atomicMax(s_max + r, e);
      else
        atomicMax(x_exp + r, e);
    }
  }
  exp_block_end(nrhs, s_max, x_exp);
}

// Batch versions: block i handles rows [row0, row0 + nrows) of one problem
// (tasks built on the host), its warps taking groups of rows.
__global__ void x_exponent_batch_kernel(const PrepProblem *probs, const PrepTask *tasks) {
  __shared__ int s_max[kExpSmemRhs];
  const PrepTask t = tasks[blockIdx.x];
  const PrepProblem &P = probs[t.problem];
  exp_block_begin(P.nrhs, s_max);
  const int lane = threadIdx.x & 31;
  for (int i = (threadIdx.x >> 5) * kRowGroup; i < t.nrows; i += (blockDim.x >> 5) * kRowGroup)
    group_exponent_max(P.d, P.tr, P.coefs, P.nrhs, P.x_exp, t.row0 + i,
                       min(kRowGroup, t.nrows - i), lane, s_max);
  exp_block_end(P.nrhs, s_max, P.x_exp);
}

// Dynamic shared memory: (blockDim.x / 32) x kPlaneGroup x (largest kp) * 8 bytes.
__global__ void __launch_bounds__(128)
    x_planes_batch_kernel(const PrepProblem *probs, const PrepTask *tasks, int max_row_bytes) {
  extern __shared__ __align__(16) uint8_t s_stage[];
  const PrepTask t = tasks[blockIdx.x];
  const PrepProblem &P = probs[t.problem];
  const int lane = threadIdx.x & 31;
  uint8_t *stage = s_stage + (threadIdx.x >> 5) * kPlaneGroup * max_row_bytes;
  for (int i = (threadIdx.x >> 5) * kPlaneGroup; i < t.nrows;
       i += (blockDim.x >> 5) * kPlaneGroup)
    group_planes<kPlaneGroup>(P.d, P.tr, P.coefs, P.nrhs, P.x_exp, P.xpl, P.kp, P.kc, P.st,
                              t.row0 + i, min(kPlaneGroup, t.nrows - i), lane, stage);
}

// 2D log displacement: w[b, r] = dispfac(b) * sum_s nmlz[lev(b), s] * coef
// (complex when the normalizers are), then disp[tb, r] = sum over list 1.
__device__ __forceinline__ void disp_box_row(const DevDesc &d, const TreeDev &tr,
                                             const double *coefs, int nrhs, double *w,
                                             int64_t idx) {
  const int cv = d.table_cplx ? 2 : 1;
  const int b = (int)(idx / nrhs), r = (int)(idx % nrhs);
  double re = 0.0, im = 0.0;
  int cnt = min(tr.src_counts[b], d.nq);
  if (cnt > 0) {
    const int lvl = tr.levels[b];
    const double ext = level_extent(tr.root_extent, lvl);
    const double f = __dmul_rn(__dmul_rn(d.disp_coef, pair_scaling(d, ext)),
                               log(__ddiv_rn(ext, d.table_root_extent)));
    const int lev = pair_table_level(d, lvl);
    const double *c = coefs + (int64_t)r * tr.n_particles + tr.src_starts[b];
    for (int s = 0; s < cnt; ++s) {
      const int64_t ni = (int64_t)lev * d.nq + s;
      re += c[s] * (f * (d.table_cplx ? d.nmlz[2 * ni] : d.nmlz[ni]));
      if (d.table_cplx) im += c[s] * (f * d.nmlz[2 * ni + 1]);
    }
  }
  w[idx * cv] = re;
  if (cv == 2) w[idx * cv + 1] = im;
}

__device__ __forceinline__ void disp_target_row(const DevDesc &d, const TreeDev &tr, int nrhs,
                                                const double *w, double *disp, int64_t idx) {
  const int cv = d.table_cplx ? 2 : 1;
  const int tb = (int)(idx / nrhs), r = (int)(idx % nrhs);
  double re = 0.0, im = 0.0;
  for (int p = tr.starts[tb]; p < tr.starts[tb + 1]; ++p) {
    const int64_t wi = ((int64_t)tr.lists[p] * nrhs + r) * cv;
    re += w[wi];
    if (cv == 2) im += w[wi + 1];
  }
  disp[idx * cv] = re;
  if (cv == 2) disp[idx * cv + 1] = im;
}

__global__ void disp_box_kernel(DevDesc d, TreeDev tr, int nboxes, const double *coefs,
                                int nrhs, double *w) {
  const int64_t n = (int64_t)nboxes * nrhs;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x)
    disp_box_row(d, tr, coefs, nrhs, w, idx);
}

__global__ void disp_target_kernel(DevDesc d, TreeDev tr, int nrhs, const double *w,
                                   double *disp) {
  const int64_t n = (int64_t)tr.n_tgt_boxes * nrhs;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x)
    disp_target_row(d, tr, nrhs, w, disp, idx);
}

// batch versions over the density-row and target-row task lists (problems
// without a displacement return at once)
__global__ void disp_box_batch_kernel(const PrepProblem *probs, const PrepTask *tasks) {
  const PrepTask t = tasks[blockIdx.x];
  const PrepProblem &P = probs[t.problem];
  if (!P.wbox) return;
  for (int i = threadIdx.x; i < t.nrows; i += blockDim.x)
    disp_box_row(P.d, P.tr, P.coefs, P.nrhs, P.wbox, t.row0 + i);
}

__global__ void disp_target_batch_kernel(const PrepProblem *probs, const PrepTask *tasks) {
  const PrepTask t = tasks[blockIdx.x];
  const PrepProblem &P = probs[t.problem];
  if (!P.disp) return;
  for (int i = threadIdx.x; i < t.nrows; i += blockDim.x)
    disp_target_row(P.d, P.tr, P.nrhs, P.wbox, P.disp, t.row0 + i);
}

// v * 2^k rounded once to FP64 (nearest, ties to even), with integer
// operations only while the result is a normal number
__device__ __forceinline__ double scaled_i64_to_double(long long v, int k) {
  if (v == 0) return 0.0;
  const unsigned long long sgn = v < 0 ? (1ull << 63) : 0ull;
  const unsigned long long mag =
      v < 0 ? (unsigned long long)(-(v + 1)) + 1ull : (unsigned long long)v;
  const int lz = __clzll((long long)mag);
  const unsigned long long m = mag << lz;   // leading one at bit 63
  unsigned long long frac = m >> 11;        // 53 significant bits
  const unsigned long long rem = m & 0x7FFull;
  int ex = 63 - lz + k;                     // v * 2^k = (m / 2^63) * 2^ex
  if (rem > 0x400ull || (rem == 0x400ull && (frac & 1ull))) {
    ++frac;
    if (frac == (1ull << 53)) {
      frac >>= 1;
      ++ex;
    }
  }
  const int biased = ex + 1023;
  if (biased >= 1 && biased <= 2046)
    return __longlong_as_double((long long)(sgn | ((unsigned long long)biased << 52) |
                                            (frac & 0xFFFFFFFFFFFFFull)));
  return ldexp((double)v, k);   // subnormal or overflowing results
}

// round(x * 2^s) to the nearest int64 for a tail accumulator x (|x| * 2^s
// below 2^62), with 32-bit conversions only (64-bit conversions run on the
// narrow FP64 side of this GPU): h = trunc(x * 2^s / 2^31) is exact in
// FP32, the remainder x * 2^s - h * 2^31 (one FMA, exact: it is the low bits
// of x's 24-bit significand) is below 2^31 in magnitude and rounds to
// nearest in one conversion.
__device__ __forceinline__ long long f32_scaled_to_i64(float x, float two_s) {
  const float xs = x * two_s;                        // exact: a power of two
  const float h = truncf(xs * 4.656612873077393e-10f);   // x * 2^s / 2^31, toward 0
  const float rem = __fmaf_rn(-h, 2147483648.0f, xs);     // exact
  return ((long long)__float2int_rz(h) << 31) + (long long)__float2int_rn(rem);
}

// ---------------------------------------------------------- main kernel

struct MixedParams {
  DevDesc d;
  MixedGeom g;
  int nrhs;
  vl1_mixed_schedule sched;
  const __half *xpl;     // density digit planes [n_xrows][n_kc][4][kc]
  int32_t n_xrows;
  const __half *adig;
  const int *x_exp;     // per rhs: kExpBias + the densities' scale exponent
  int a_exp;
  const double *disp;  // [n_tgt_boxes * nrhs] (x2 complex) or nullptr
  const int32_t *target_boxes, *tgt_starts, *tgt_counts;
  int n_tgt_boxes;
  int64_t n_particles;
  double *result;
  vl1_status *st;
  // bounded waits: microseconds before a wait gives up (0: kWaitLimitUs);
  // test hook (vl1_test_set_wait_fault): when nonzero, producer warp 0 of CTA
  // (0, 0) withholds its arrival for that CTA's first pipeline unit, so that
  // the tensor-core issuer's wait runs out and the launch reports
  // VL1_E_TIMEOUT
  uint32_t wait_limit_us;
  int32_t withhold_arrival;
};

// Warp roles of mixed_kernel (warp index w):
//   w <  8      producers: per pipeline unit, warp w copies the density digit
//               planes of tile rows 16w .. 16w+15 into the unit's stage with
//               cp.async (16-byte pieces straight into the swizzled K-major
//               layout, zero-filled for rows without a source box); each
//               lane's arrival on xfull[stage] fires when its copies land
//               (cp.async.mbarrier.arrive), so the producers never wait for
//               data, only for a free stage.  Eight warps keep enough
//               requests in flight to cover the L2 latency of these scattered
//               rows.
//   w == 8      table loader (one lane): the five table digit tiles of the
//               unit's key by bulk copies (TMA), counted on afull[stage]
//   w == 9      tensor-core issuer (one lane)
//   w >= 10     readout: TMEM lane quadrant w % 4, RC columns each
// Pipeline unit = (key, K chunk of kc <= 32 source points); a "round" = the
// consecutive units (of one or more keys) that share an exact accumulation
// (K <= kRoundK = 128).  Exact
// diagonal accumulators (i+j = 2, 3, 4) are double-buffered in TMEM (one
// buffer per round parity) so the readout of round r overlaps the products of
// round r+1; the tail diagonals (i+j = 5, 6) accumulate over the whole tile.
// The table digit planes j = 1..5 of a stage are stacked along N, so one MMA
// multiplies density digit i by several table digits j at once; its output
// column blocks land on consecutive diagonals i + j.
// Density planes of a stage: the exact digits X1, X2, X3 and, for the tails
// only, R = X4 + X5 / 256 rounded to FP16 (11 significant bits: the density
// keeps ~2^-36 of its rhs's scale in the tails, far below the 2^-24 weight of
// the tails; the exact diagonals use X1..X3 only).
// Roles and pipeline depth per column chunk width.  64 output columns: 8
// producer warps, 4 stages, one CTA per SM (214 KB of shared memory, all 512
// TMEM columns).  16 or 32 columns: 4 producer warps, 2 stages and two CTAs
// per SM (at most 91 KB and 256 TMEM columns each, <= 73 registers per
// thread), so that one CTA's pipeline fill, readout and result write overlap
// the other's tensor-core work.
template <int NCH>
struct MixedRoles {
  static constexpr int kProducers = NCH >= 64 ? 8 : 4;
  static constexpr int kRowsPerProducer = 128 / kProducers;
  static constexpr int kLoader = kProducers;
  static constexpr int kMma = kProducers + 1;
  static constexpr int kRead0 = kProducers + 2;
  static constexpr int kStages = NCH >= 64 ? 4 : 2;
  static constexpr int kCtasPerSm = NCH >= 64 ? 1 : 2;
  static constexpr int kThreads = 32 * (kRead0 + 4 * (NCH / 16));
};
constexpr int kMaxStages = 4;
// source points of one exact round: with balanced digits (|digit| <= 128) a
// diagonal sum over 128 points is at most 2^21 (i + j = 2), 2^22 (i + j = 3)
// and 3 * 2^21 (i + j = 4), all exact in FP32
constexpr int kRoundK = 128;
constexpr uint32_t kExactCols = 3;   // accumulators per buffer
constexpr uint32_t kSleepNs = 200000;      // suspend hint of one barrier test
constexpr uint32_t kWaitLimitUs = 2000000; // a wait gives up after 2 s
// split-tile counters: parts in the low 16 bits, aborted parts also in the
// high bits (a tile has fewer than 2^16 parts)
constexpr int kSplitPoison = 1 << 16;
// split counters are spaced 16 apart (one per split tile and column chunk,
// in a layout that leaves room for per-piece counts)
constexpr int kSplitCounterStride = 16;

struct Barriers {
  uint64_t xfull[kMaxStages];   // every producer lane's density copies have landed
  uint64_t afull[kMaxStages];   // the table digit tiles have landed
  uint64_t empty[kMaxStages];
  uint64_t accf[2];
  uint64_t acce[2];
  uint64_t drain;            // after an abort: every issued MMA has completed
};

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Wait for `phase` of `bar`.  Gives up (returns false) when another role has
// set the abort flag, or after `limit_us` microseconds (then it sets the
// flag itself); both are looked at every 32 tests.  A warp whose test fails
// sleeps between tests, so that waiting warps leave the issue slots of
// their scheduler to the producer warps that share it: with `backoff` the
// sleep doubles from 32 ns to 256 ns (warps with slack: producers, readout);
// without it, it stays at 32 ns (the tensor-core issuer and the table
// loader, whose reaction time is on the pipeline's critical path).
__device__ __forceinline__ bool wait_or_abort(uint64_t *bar, uint32_t phase,
                                              volatile int *abort_flag, uint32_t limit_us,
                                              bool backoff) {
  if (tc::mbar_try_wait_sleep(bar, phase, kSleepNs)) return true;
  const uint64_t t0 = global_ns();
  uint32_t ns = 32;
  for (uint32_t i = 1;; ++i) {
    __nanosleep(ns);
    if (backoff) ns = ns < 256 ? 2 * ns : ns;
    if (tc::mbar_try_wait_sleep(bar, phase, kSleepNs)) return true;
    if ((i & 31u) == 0u) {
      if (*abort_flag) return false;
      if (global_ns() - t0 > (uint64_t)limit_us * 1000ull) break;
    }
  }
  *abort_flag = 1;
  return false;
}

// Wait for `phase` of `bar` regardless of the abort flag, at most
// `limit_us`: used after an abort for operations already issued (bulk copies
// into this CTA's shared memory, MMAs into its TMEM), which complete on
// their own, before the CTA releases its TMEM and exits.
__device__ __forceinline__ bool wait_bounded(uint64_t *bar, uint32_t phase, uint32_t limit_us) {
  const uint64_t t0 = global_ns();
  while (!tc::mbar_try_wait_sleep(bar, phase, kSleepNs)) {
    if (global_ns() - t0 > (uint64_t)limit_us * 1000ull) return false;
    __nanosleep(256);
  }
  return true;
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_addr(bar)) : "memory");
}

// A work item of a batch launch: one problem's tile (or key range of it) and
// output column chunk.
struct BatchItem {
  int32_t problem, chunk;
  vl1_mixed_item item;
};
struct BatchLaunch {
  const MixedParams *probs;   // [n_problems]
  const BatchItem *items;     // [n_items], launched in this order
  int n_items;
  int *queue;                 // next item to take; zero before the launch
  uint32_t wait_limit_us;     // as MixedParams::wait_limit_us (persistent launches)
  int32_t withhold_arrival;   // as MixedParams::withhold_arrival
};

// One group of MMAs: density digit i times the stacked table digits
// j0 .. j0 + nb - 1, into nb consecutive diagonal blocks.
struct MmaGroup {
  int i, j0, nb, exact;  // exact: into the round buffer (else the tail blocks)
};
// exact diagonals 2..4: (1; 1..3), (2; 1..2), (3; 1); tails 5..6:
// (1; 4..5), (2; 3..4), (3; 2..3), (R; 1..2) with density plane 4 holding
// R = X4 + X5 / 256: R A1 = X4 A1 + X5 A1 / 256 covers (4, 1) and (5, 1),
// R A2 covers (4, 2) (plus the negligible (5, 2) / 256)
constexpr int kGroupCount = 7;
__device__ constexpr MmaGroup kGroups[kGroupCount] = {{1, 1, 3, 1}, {2, 1, 2, 1}, {3, 1, 1, 1},
                                                      {1, 4, 2, 0}, {2, 3, 2, 0}, {3, 2, 2, 0},
                                                      {4, 1, 2, 0}};

// MULTI == false: one work item per CTA (blockIdx.x; column chunk blockIdx.y)
// of the single problem p1.  MULTI == true: a persistent launch over the
// items of several problems, each CTA taking the next item from bl.queue; the
// item's problem parameters are copied to shared memory, and the pipeline
// barriers keep their phases across items (CTA-wide unit / round counters).
template <int NCH, int KC, bool MULTI>
__global__ void __launch_bounds__(MixedRoles<NCH>::kThreads, MixedRoles<NCH>::kCtasPerSm)
mixed_kernel(const __grid_constant__ MixedParams p1, const __grid_constant__ BatchLaunch bl) {
  using Roles = MixedRoles<NCH>;
  constexpr int kStages = Roles::kStages;
  constexpr int kProducerWarps = Roles::kProducers;
  constexpr int kRowsPerProducer = Roles::kRowsPerProducer;
  constexpr int kLoaderWarp = Roles::kLoader;
  constexpr int kMmaWarp = Roles::kMma;
  constexpr int kReadWarp0 = Roles::kRead0;
  constexpr int RC = 16;                            // columns per readout warp
  constexpr int NREAD = 4 * (NCH / RC);             // readout warps
  // TMEM: [buffer 0: 3 x NCH][tail d5][tail d6][buffer 1: 3 x NCH]
  constexpr uint32_t COLS = NCH * 8 > 256 ? 512 : (NCH * 8 > 128 ? 256 : 128);
  constexpr uint32_t XBYTES = 128u * KC * 2u;      // one digit plane of the rows
  constexpr uint32_t ABYTES = (uint32_t)NCH * KC * 2u;   // one digit plane of the table
  constexpr uint32_t STAGE_BYTES = kXPlanes * XBYTES + kDigits * ABYTES;
  constexpr uint32_t ROW_BYTES = KC * 2u;
  // parked int64 sums: rows padded by one value, so that the 32 lanes of a
  // readout warp (32 rows) store one column into distinct banks
  constexpr int PARK_STRIDE = NCH + 1;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  // swizzle atoms need a 1024-byte aligned base (the launch adds 1 KiB slack)
  uint8_t *smem = reinterpret_cast<uint8_t *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  __shared__ Barriers bars;
  __shared__ uint32_t tmem_base;
  __shared__ volatile int s_abort;
  __shared__ int s_rows[128];
  __shared__ __align__(16) MixedParams s_p;   // MULTI: the current item's problem
  __shared__ int s_next;
  const MixedParams &p = MULTI ? s_p : p1;

  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int lane = tid & 31;
  const uint32_t lim = MULTI ? bl.wait_limit_us : p1.wait_limit_us;
  const uint32_t limit_us = lim ? lim : kWaitLimitUs;
  // test hook: this CTA's producer warp 0 withholds its first arrival
  const bool withhold = (MULTI ? bl.withhold_arrival : p1.withhold_arrival) != 0 &&
                        blockIdx.x == 0 && blockIdx.y == 0;

  if (tid == 0) {
    tc::mbar_init(&bars.drain, 1);
    for (int s = 0; s < kStages; ++s) {
      tc::mbar_init(&bars.xfull[s], kProducerWarps * 32);   // one per producer lane
      tc::mbar_init(&bars.afull[s], 1);                // the loader's expect_tx
      tc::mbar_init(&bars.empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(&bars.accf[b], 1);
      tc::mbar_init(&bars.acce[b], NREAD);
    }
    tc::fence_mbar_init();
    s_abort = 0;
  }
  if (warp == kMmaWarp) {
    tc::tmem_alloc(&tmem_base, COLS);
    tc::tmem_relinquish();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tbase = tmem_base;

  // pipeline units and K rounds this CTA has run in earlier items (stage and
  // buffer phases continue across items)
  int ubase = 0, rbase = 0;
  for (int pass = 0;; ++pass) {
  int wi;
  if (MULTI) {
    if (tid == 0) s_next = s_abort ? bl.n_items : atomicAdd(bl.queue, 1);
    __syncthreads();
    wi = s_next;
    if (wi >= bl.n_items) break;
    const uint64_t *src = reinterpret_cast<const uint64_t *>(bl.probs + bl.items[wi].problem);
    for (int i = tid; i < (int)(sizeof(MixedParams) / 8); i += blockDim.x)
      reinterpret_cast<uint64_t *>(&s_p)[i] = src[i];
    __syncthreads();
  } else {
    if (pass > 0) break;
    wi = blockIdx.x;
  }
  const int chunk = MULTI ? bl.items[wi].chunk : blockIdx.y;
  const int n_chunks = p.g.np / NCH;

  // this CTA's work item: a tile, or a key range of a split tile
  vl1_mixed_item item;
  if (MULTI) {
    item = bl.items[wi].item;
  } else if (p.sched.n_items > 0) {
    item = p.sched.items[wi];
  } else {
    item.tile = wi;
    item.key_begin = p.sched.tile_key_start[wi];
    item.key_end = p.sched.tile_key_start[wi + 1];
    item.split = -1;
    item.part = 0;
    item.nparts = 1;
    item.slot = -1;
  }
  const int tile = item.tile;
  {
    bool bad = tile < 0 || tile >= p.sched.n_tiles || chunk < 0 || chunk >= n_chunks;
    if (!bad) {
      const int t0 = p.sched.tile_key_start[tile], t1 = p.sched.tile_key_start[tile + 1];
      bad = item.key_begin < t0 || item.key_end > t1 || item.key_begin > item.key_end;
    }
    if (item.split >= 0)
      bad = bad || item.split >= p.sched.n_splits || item.part < 0 ||
            item.part >= item.nparts || item.nparts >= kSplitPoison ||
            item.slot - item.part < 0 ||
            item.slot - item.part + item.nparts > p.sched.n_slots;
    else
      bad = bad || item.split != -1;
    if (bad) {   // uniform across the CTA
      if (tid == 0) report(p.st, VL1_E_ARG, wi, -1);
      __syncthreads();
      continue;
    }
  }

  const int k0 = item.key_begin, k1 = item.key_end;
  const int n_keys = k1 - k0;
  // units of the item, and exact rounds of up to kRoundK source points (a
  // round may span several keys: the exact diagonals of every key of a tile
  // row are in the same units)
  const int n_units = n_keys * p.g.n_kc;
  constexpr int upr = kRoundK / KC;   // units per round
  const int n_rounds = (n_units + upr - 1) / upr;

  // the rows of the tile, and (for the result write at the end of the item,
  // loaded now so that their latency hides behind the pipeline) each row's
  // first result index, point count and output exponent
  __shared__ long long s_obase[128];   // result index of the row's first target point
  __shared__ int s_ocnt[128];          // target points of the row's box (0: empty row)
  __shared__ int s_oexp[128];          // an output is (parked sum) * 2^s_oexp
  if (tid < 128) {
    int v = p.sched.tile_rows[(int64_t)tile * 128 + tid];
    if (v >= (int64_t)p.n_tgt_boxes * p.nrhs) {
      report(p.st, VL1_E_ARG, tile, tid);
      v = -1;
    }
    s_rows[tid] = v;
    int cnt = 0, ex = 0;
    long long ob = 0;
    if (v >= 0) {
      const int j = v / p.nrhs, r = v - (v / p.nrhs) * p.nrhs;
      const int tbox = p.target_boxes[j];
      cnt = min(p.tgt_counts[tbox], p.d.nq);
      ob = (long long)r * p.n_particles + p.tgt_starts[tbox];
      // table values are m_a 2^(a_exp - kFixedBits), densities
      // m_x 2^(e - kXFixedBits) with e the scale exponent of the rhs; the
      // parked sums count units of 2^32 of m_a m_x
      ex = p.a_exp + (p.x_exp[r] - kExpBias) - (kFixedBits + kXFixedBits) + 32;
    }
    s_obase[tid] = ob;
    s_ocnt[tid] = cnt;
    s_oexp[tid] = ex;
  }
  __syncthreads();

  if (warp < kProducerWarps) {
    // ------------------------------------------------------------ producers
    // Per unit: wait for the unit's stage to be free, then copy the four
    // digit planes of this warp's 16 rows (8 * KC bytes of a row: PPR 16-byte
    // pieces of 8 values of one plane) into the stage's swizzled K-major
    // planes with cp.async; each lane's arrival on xfull fires when its own
    // copies have landed.  A warp none of whose rows has a source box in the
    // unit's key writes zero planes (once per stage) and arrives at once.
    constexpr int PPP = KC / 8;                          // pieces per row and plane
    constexpr int PPR = kXPlanes * PPP;                  // pieces per row and unit
    constexpr int NIT = kRowsPerProducer * PPR / 32;     // pieces per lane and unit
    static_assert(kRowsPerProducer * PPR % 32 == 0, "whole pieces per lane");
    const int64_t row_halves = (int64_t)p.g.kp * kXPlanes;   // FP16 values per density row
    // lanes < kRowsPerProducer hold the density row of tile row my_row,
    // fetched one key ahead
    const int my_row = kRowsPerProducer * warp + (lane % kRowsPerProducer);
    int nkey = 0, nxr = -1;
    if (n_keys > 0) {
      nkey = p.sched.key_ids[k0];
      nxr = p.sched.key_xrow[(int64_t)k0 * 128 + my_row];
    }
    // bit s: this warp's rows of stage s hold zero planes (the stages are
    // overwritten by the parked sums at the end of an item, so the bits
    // start clear per item)
    uint32_t zero_stages = 0;
    int u = 0;
    bool aborted = false;
    for (int kidx = k0; kidx < k1 && !aborted; ++kidx) {
      const int key = nkey;
      int xr_lane = nxr;
      if (kidx + 1 < k1) {
        nkey = p.sched.key_ids[kidx + 1];
        nxr = p.sched.key_xrow[(int64_t)(kidx + 1) * 128 + my_row];
      }
      const bool key_ok = key >= 0 && key < p.d.n_tables * p.d.n_cases;
      if (!key_ok) {
        if (warp == 0 && lane == 0) report(p.st, VL1_E_ARG, tile, kidx);
        xr_lane = -1;
      }
      if (xr_lane >= p.n_xrows) {
        report(p.st, VL1_E_ARG, tile, my_row);
        xr_lane = -1;
      }
      const bool key_empty =
          __ballot_sync(0xffffffffu, lane < kRowsPerProducer && xr_lane >= 0) == 0u;
      for (int kc = 0; kc < p.g.n_kc; ++kc, ++u) {
        const int s = (ubase + u) % kStages;
        const int use = (ubase + u) / kStages;
        if (use > 0 &&
            !wait_or_abort(&bars.empty[s], (use - 1) & 1, &s_abort, limit_us, true)) {
          aborted = true;
          break;
        }
        uint8_t *xs = smem + (size_t)s * STAGE_BYTES;
        const bool hold = withhold && warp == 0 && ubase + u == 0;
        if (key_empty) {
          // no source rows: zero planes (rows 16w .. 16w + 15 of a swizzled
          // K-major plane are one contiguous block), written once per stage
          if (!((zero_stages >> s) & 1u)) {
            constexpr int BLK = kRowsPerProducer * (int)ROW_BYTES;
#pragma unroll
            for (int dg = 0; dg < kXPlanes; ++dg)
              for (int o = lane * 16; o < BLK; o += 32 * 16)
                *reinterpret_cast<uint4 *>(xs + dg * XBYTES + warp * BLK + o) =
                    make_uint4(0u, 0u, 0u, 0u);
            zero_stages |= 1u << s;
          }
          tc::fence_proxy_async_smem();
          __syncwarp();
          if (!hold) mbar_arrive(&bars.xfull[s]);
          continue;
        }
        zero_stages &= ~(1u << s);
#pragma unroll
        for (int it = 0; it < NIT; ++it) {
          // piece pc of the warp's rows: row pc / PPR, plane q / PPP, values
          // 8 (q % PPP) .. +7 of the K chunk (consecutive lanes read one
          // row's 8 * KC contiguous bytes)
          const int pc = it * 32 + lane;
          const int rl = pc / PPR, q = pc - (pc / PPR) * PPR;
          const int pl = q / PPP, k8 = q - (q / PPP) * PPP;
          const int xr = __shfl_sync(0xffffffffu, xr_lane, rl);
          const int row = kRowsPerProducer * warp + rl;
          const bool have = xr >= 0;
          const __half *src =
              p.xpl + (have ? (int64_t)xr * row_halves + ((int64_t)kc * kXPlanes + pl) * KC +
                                  k8 * 8
                            : 0);
          tc::cp_async16_zfill(xs + pl * XBYTES + tc::kmajor_swizzled_offset(row, k8 * 8, KC),
                               src, have ? 16u : 0u);
        }
        if (!hold) tc::cp_async_mbar_arrive_noinc(&bars.xfull[s]);
      }
    }
    tc::cp_async_wait_all();
    __syncwarp();
  } else if (warp == kLoaderWarp) {
    // ---------------------------------------------------------- table loader
    if (lane == 0) {
      int u = 0;
      bool aborted = false;
      int nkey = n_keys > 0 ? p.sched.key_ids[k0] : 0;
      for (int kidx = k0; kidx < k1 && !aborted; ++kidx) {
        int key = nkey;
        if (kidx + 1 < k1) nkey = p.sched.key_ids[kidx + 1];
        if (key < 0 || key >= p.d.n_tables * p.d.n_cases) key = 0;   // reported by warp 0
        for (int kc = 0; kc < p.g.n_kc; ++kc, ++u) {
          const int s = (ubase + u) % kStages;
          const int use = (ubase + u) / kStages;
          if (use > 0 &&
              !wait_or_abort(&bars.empty[s], (use - 1) & 1, &s_abort, limit_us, false)) {
            aborted = true;
            break;
          }
          uint8_t *as = smem + (size_t)s * STAGE_BYTES + kXPlanes * XBYTES;
          tc::mbar_arrive_expect_tx(&bars.afull[s], kDigits * ABYTES);
          const int64_t base = (((int64_t)key * p.g.n_kc + kc) * kDigits) * p.g.np * KC +
                               (int64_t)chunk * NCH * KC;
          if (n_chunks == 1) {
            // one column chunk: the five digit tiles are contiguous
            tc::bulk_g2s(as, p.adig + base, kDigits * ABYTES, &bars.afull[s]);
          } else {
#pragma unroll
            for (int dg = 0; dg < kDigits; ++dg)
              tc::bulk_g2s(as + dg * ABYTES, p.adig + base + (int64_t)dg * p.g.np * KC, ABYTES,
                           &bars.afull[s]);
          }
        }
      }
      if (aborted || s_abort) {
        // copies of the last (up to kStages) issued units may still be in
        // flight into this CTA's stages: let them land before the CTA exits
        for (int v = u - kStages < 0 ? 0 : u - kStages; v < u; ++v)
          wait_bounded(&bars.afull[(ubase + v) % kStages], ((ubase + v) / kStages) & 1,
                       limit_us);
      }
    }
    __syncwarp();
  } else if (warp == kMmaWarp) {
    // ------------------------------------------------------- tensor cores
    if (lane == 0) {
      const uint32_t tail_col = tbase + kExactCols * NCH;
      int u = 0;
      bool aborted = false;
      for (int round = 0; round < n_rounds && !aborted; ++round) {
        const int R = rbase + round;
        const int b = R & 1;
        if (R >= 2 &&
            !wait_or_abort(&bars.acce[b], ((R >> 1) - 1) & 1, &s_abort, limit_us, false)) {
          aborted = true;
          break;
        }
        tc::tc_fence_after();
        const uint32_t exact_col = tbase + (uint32_t)b * 5 * NCH;
        for (int iu = 0; iu < upr && u < n_units; ++iu, ++u) {
          const int s = (ubase + u) % kStages;
          const uint32_t ph = ((ubase + u) / kStages) & 1;
          if (!wait_or_abort(&bars.afull[s], ph, &s_abort, limit_us, false)) {
            aborted = true;
            break;
          }
          if (!wait_or_abort(&bars.xfull[s], ph, &s_abort, limit_us, false)) {
            aborted = true;
            break;
          }
          // the digit rows were written by cp.async (generic proxy): order
          // them before the tensor cores' (async proxy) reads
          tc::fence_proxy_async_smem();
          tc::tc_fence_after();
          const uint32_t xa = tc::smem_addr(smem + (size_t)s * STAGE_BYTES);
          // descriptors advance by (byte offset >> 4) in their address field
          const uint64_t xd = tc::smem_desc_kmajor_swizzled(xa, ROW_BYTES);
          const uint64_t adsc = tc::smem_desc_kmajor_swizzled(xa + kXPlanes * XBYTES, ROW_BYTES);
#pragma unroll
          for (int kk = 0; kk < KC / 16; ++kk) {
#pragma unroll
            for (int g = 0; g < kGroupCount; ++g) {
              const MmaGroup gr = kGroups[g];
              const uint32_t col = gr.exact ? exact_col + (uint32_t)(gr.i + gr.j0 - 2) * NCH
                                            : tail_col + (uint32_t)(gr.i + gr.j0 - 5) * NCH;
              const bool first = gr.exact ? (g == 0 && iu == 0 && kk == 0)
                                          : (g == 3 && u == 0 && kk == 0);
              const uint64_t ad = xd + (((uint32_t)(gr.i - 1) * XBYTES + kk * 32u) >> 4);
              const uint64_t bd = adsc + (((uint32_t)(gr.j0 - 1) * ABYTES + kk * 32u) >> 4);
              tc::mma_f16(col, ad, bd, tc::idesc_f16_f32(128, NCH * gr.nb), first ? 0u : 1u);
            }
          }
          tc::mma_commit(&bars.empty[s]);   // stage free once these products finish
        }
        if (!aborted) tc::mma_commit(&bars.accf[b]);
      }
      if (aborted || s_abort) {
        // MMAs issued before the abort still write TMEM and read the stages:
        // wait for all of them before the TMEM is released
        tc::mma_commit(&bars.drain);
        wait_bounded(&bars.drain, 0, limit_us);
      }
    }
    __syncwarp();
  } else {
    // ------------------------------------------------------------ readout
    const int rw = warp - kReadWarp0;      // 0 .. NREAD-1
    const int quad = warp & 3;             // TMEM lanes 32*quad .. +31
    const int cb = rw >> 2;                // RC-column block
    const uint32_t lane_off = (uint32_t)(quad * 32) << 16;
    const int row = quad * 32 + lane;
    // exact sum of the diagonals per output, units of 2^(e-32); the d = 2
    // and d = 3 terms enter as the raw bits of (d + 1.5 * 2^23), whose
    // constant part is taken out once after the loop
    unsigned long long acc[RC];
#pragma unroll
    for (int c = 0; c < RC; ++c) acc[c] = 0;
    bool ok = true;
    int rounds_read = 0;
    for (int round = 0; round < n_rounds; ++round) {
      const int R = rbase + round;
      const int b = R & 1;
      if (!wait_or_abort(&bars.accf[b], (R >> 1) & 1, &s_abort, limit_us, true)) {
        ok = false;
        break;
      }
      tc::tc_fence_after();
      const uint32_t col = tbase + lane_off + (uint32_t)b * 5 * NCH + cb * RC;
      uint32_t r2[16], r3[16];
      tc::tmem_ld16(col, r2);                // i + j = 2: |x| <= 128 * 128 * 128 = 2^21
      tc::tmem_ld16(col + NCH, r3);          // i + j = 3: |x| <= 2 * 2^21 = 2^22
      tc::tmem_ld_wait();
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        // 1.5 * 2^23 + x for |x| <= 2^22 is exact and its raw bits are
        // kMagicBits + x (also at x = 2^22, where the sum is 2^24); weights
        // 2^16 and 2^8 of the d = 2 and d = 3 terms
        const uint32_t b2 = __float_as_uint(__uint_as_float(r2[c]) + kMagic);
        const uint32_t b3 = __float_as_uint(__uint_as_float(r3[c]) + kMagic);
        acc[c] += (unsigned long long)b2 * 65536ull + (unsigned long long)b3 * 256ull;
      }
      tc::tmem_ld16(col + 2 * NCH, r2);      // i + j = 4: |x| <= 3 * 2^21 < 2^24
      tc::tmem_ld_wait();
      tc::tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&bars.acce[b]);
#pragma unroll
      for (int c = 0; c < 16; ++c)
        acc[c] += (unsigned long long)(long long)__float2int_rn(__uint_as_float(r2[c]));
      ++rounds_read;
    }
    // ---- park one int64 per output: the sum of digit products in units of
    // 2^32 (integer diagonals 2..4, weights 2^64..2^48, shifted by 16, plus
    // the FP32 tails d5, d6 of weights 2^40, 2^32 rounded to that unit)
    if (ok && !s_abort) {
      long long *s_tot = reinterpret_cast<long long *>(smem);
      const uint32_t col = tbase + lane_off + kExactCols * NCH + cb * RC;
      // the constant parts of the raw bits, (kMagicBits << 16) + (kMagicBits
      // << 8) per round (modulo 2^64: the true sum fits an int64)
      const unsigned long long magic_total =
          (unsigned long long)rounds_read * ((unsigned long long)kMagicBits * 65792ull);
#pragma unroll
      for (int c = 0; c < 16; ++c) acc[c] = (acc[c] - magic_total) << 16;
      if (n_rounds > 0) {
        uint32_t r16[16];
        tc::tmem_ld16(col, r16);                 // d5, weight 2^40
        tc::tmem_ld_wait();
#pragma unroll
        for (int c = 0; c < 16; ++c)
          acc[c] += (unsigned long long)f32_scaled_to_i64(__uint_as_float(r16[c]), 256.0f);
        tc::tmem_ld16(col + NCH, r16);           // d6, weight 2^32
        tc::tmem_ld_wait();
#pragma unroll
        for (int c = 0; c < 16; ++c)
          acc[c] += (unsigned long long)f32_scaled_to_i64(__uint_as_float(r16[c]), 1.0f);
      }
#pragma unroll
      for (int c = 0; c < 16; ++c)
        s_tot[row * PARK_STRIDE + cb * RC + c] = (long long)acc[c];
    }
  }

  // ---- all warps: final values and coalesced writes (a row's outputs are
  // the consecutive target points of one box).  A split tile's parts store
  // their exact partial sums; the part that finishes last adds them (exactly,
  // in int64) and writes the results.  The one rounding to FP64 is done with
  // integer operations (the FP64 pipe is narrow on this GPU).
  tc::tc_fence_before();
  __syncthreads();
  __shared__ int s_last, s_poison;
  const long long *tot_src = reinterpret_cast<const long long *>(smem);
  bool write = !s_abort;
  // a split tile's accumulator: the parts add their exact int64 sums into
  // the slot of part 0 (integer addition: the total does not depend on the
  // order); the part that arrives last writes the results and clears it
  unsigned long long *g_acc = nullptr;
  const int64_t slot_bytes = (int64_t)128 * NCH * 8;
  int *g_ctr = nullptr;
  if (item.split >= 0) {
    g_acc = reinterpret_cast<unsigned long long *>(
        static_cast<uint8_t *>(p.sched.split_partials) +
        ((int64_t)(item.slot - item.part) * n_chunks + chunk) * slot_bytes);
    g_ctr = p.sched.split_counters + ((int64_t)item.split * n_chunks + chunk) * kSplitCounterStride;
    if (!s_abort) {
      for (int i = tid; i < 128 * NCH; i += blockDim.x)
        atomicAdd(g_acc + i, (unsigned long long)tot_src[(i / NCH) * PARK_STRIDE + i % NCH]);
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) {
      // parts count in the low 16 bits; a part that aborted (and added no
      // sums) also adds to the high bits, so that the last part writes
      // nothing for the tile
      const int inc = s_abort ? kSplitPoison + 1 : 1;
      const int done = atomicAdd(g_ctr, inc) + inc;
      s_last = (done & (kSplitPoison - 1)) == item.nparts;
      s_poison = done >= kSplitPoison;
    }
    __syncthreads();
    write = write && s_last && !s_poison;
    if (s_last) __threadfence();
  } else {
    __syncthreads();
  }
  if (write) {
    const bool oc = p.d.table_cplx;
    // BATCH outputs per thread and pass: their loads (parked sums, or the
    // parts of a split tile from L2) are issued before any conversion
    constexpr int BATCH = 4;
    for (int it0 = tid; it0 < 128 * NCH; it0 += BATCH * (int)blockDim.x) {
      long long tot[BATCH];
#pragma unroll
      for (int bi = 0; bi < BATCH; ++bi) {
        const int it = it0 + bi * (int)blockDim.x;
        tot[bi] = 0;
        if (it >= 128 * NCH) continue;
        if (item.split >= 0) {
          tot[bi] = (long long)__ldcg(g_acc + it);
        } else {
          tot[bi] = tot_src[(it / NCH) * PARK_STRIDE + it % NCH];
        }
      }
#pragma unroll
      for (int bi = 0; bi < BATCH; ++bi) {
        const int it = it0 + bi * (int)blockDim.x;
        if (it >= 128 * NCH) continue;
        const int rw_ = it / NCH, cc = it - rw_ * NCH;
        int t = chunk * NCH + cc, part = 0;
        if (oc && t >= p.d.nq) {
          t -= p.d.nq;
          part = 1;
        }
        if (t >= s_ocnt[rw_]) continue;   // also empty rows and padding columns
        double y = scaled_i64_to_double(tot[bi], s_oexp[rw_]);
        if (p.disp) {
          const int64_t di = s_rows[rw_];   // j * nrhs + r
          y += oc ? p.disp[2 * di + part] : p.disp[di];
        }
        const int64_t o = s_obase[rw_] + t;
        if (oc)
          p.result[2 * o + part] = y;
        else
          p.result[o] = y;
      }
    }
  }
  // the last part leaves the accumulator and the counter at zero for the
  // next call (also after an abort, so that a timed-out call does not spoil
  // the schedule); each thread clears the entries it read
  if (item.split >= 0 && s_last) {
    for (int i = tid; i < 128 * NCH; i += blockDim.x) g_acc[i] = 0ull;
    if (tid == 0) *g_ctr = 0;
  }
  __syncthreads();
  if (s_abort && tid == 0) {
    report(p.st, VL1_E_TIMEOUT, tile, chunk);
    if (MULTI) {
      // the items this launch will no longer run still count their parts,
      // so that every split counter ends at zero
      for (;;) {
        const int wj = atomicAdd(bl.queue, 1);
        if (wj >= bl.n_items) break;
        const BatchItem bj = bl.items[wj];
        if (bj.item.split < 0) continue;
        const MixedParams *pj = bl.probs + bj.problem;
        const int nchk = pj->g.np / NCH;
        int *ctr = pj->sched.split_counters +
                   ((int64_t)bj.item.split * nchk + bj.chunk) * kSplitCounterStride;
        const int done = atomicAdd(ctr, kSplitPoison + 1) + kSplitPoison + 1;
        if ((done & (kSplitPoison - 1)) == bj.item.nparts) {
          // the tile's last arrival: clear what its other parts added
          unsigned long long *acc = reinterpret_cast<unsigned long long *>(
              static_cast<uint8_t *>(pj->sched.split_partials) +
              ((int64_t)(bj.item.slot - bj.item.part) * nchk + bj.chunk) * slot_bytes);
          for (int i = 0; i < 128 * NCH; ++i) acc[i] = 0ull;
          *ctr = 0;
        }
      }
    }
  }
  ubase += n_units;
  rbase += n_rounds;
  __syncthreads();
  }   // work items
  if (warp == kMmaWarp) tc::tmem_dealloc(tbase, COLS);
}

// the kernel instance for a column chunk width and K chunk (nullptr if none)
const void *mixed_kernel_ptr(int nch, int kc, bool multi) {
#define VL1_MK(N, K)                                                                   \
  if (nch == N && kc == K)                                                             \
    return multi ? reinterpret_cast<const void *>(&mixed_kernel<N, K, true>)          \
                 : reinterpret_cast<const void *>(&mixed_kernel<N, K, false>);
  VL1_MK(64, 32) VL1_MK(32, 32) VL1_MK(16, 32) VL1_MK(64, 16) VL1_MK(32, 16) VL1_MK(16, 16)
#undef VL1_MK
  return nullptr;
}

size_t mixed_smem_bytes(int nch, int kc) {
  const int stages = nch >= 64 ? MixedRoles<64>::kStages : MixedRoles<32>::kStages;
  const size_t pipe = (size_t)stages * (kXPlanes * 128 + kDigits * nch) * kc * 2;
  const size_t park = (size_t)128 * (nch + 1) * 8;   // int64 sums, padded rows
  return (pipe > park ? pipe : park) + 1024;
}

int mixed_threads(int nch) {
  return nch >= 64 ? MixedRoles<64>::kThreads
                   : (nch >= 32 ? MixedRoles<32>::kThreads : MixedRoles<16>::kThreads);
}

int mixed_ctas_per_sm(int nch) { return nch >= 64 ? 1 : 2; }

cudaError_t launch_mixed_kernel(int nch, int kc, bool multi, dim3 grid, cudaStream_t s,
                                const MixedParams &mp, const BatchLaunch &bl) {
  const void *fn = mixed_kernel_ptr(nch, kc, multi);
  if (!fn) return cudaErrorInvalidValue;
  const size_t smem = mixed_smem_bytes(nch, kc);
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  void *args[] = {const_cast<MixedParams *>(&mp), const_cast<BatchLaunch *>(&bl)};
  return cudaLaunchKernel(fn, grid, dim3(mixed_threads(nch)), args, smem, s);
}

int grid_for(int64_t n, int threads) {
  int64_t g = (n + threads - 1) / threads;
  if (g > 152 * 32) g = 152 * 32;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace

MixedGeom mixed_geometry(int nq, int table_cplx, int kc, int nch) {
  MixedGeom g;
  g.kp = ((nq + 15) / 16) * 16;
  g.kc = kc ? kc : (g.kp <= 32 ? g.kp : 32);
  // above one chunk of 32, K is padded to a multiple of 64 (whole units of
  // either K chunk)
  if (g.kp > 32) g.kp = ((g.kp + 63) / 64) * 64;
  g.n_kc = g.kp / g.kc;
  const int n = table_cplx ? 2 * nq : nq;
  g.np = ((n + 15) / 16) * 16;
  if (nch) {
    g.nch = nch;
  } else if (g.np <= 16) {
    g.nch = 16;
  } else if (g.np <= 32) {
    g.nch = 32;
  } else {
    g.nch = 64;
  }
  g.np = ((g.np + g.nch - 1) / g.nch) * g.nch;
  return g;
}

int32_t build_mixed_operands(vl1_plan *plan, double table_absmax, cudaStream_t s) {
  const DevDesc &d = plan->d;
  const MixedGeom g = plan->mixed.geom;
  plan->mixed.table_absmax = table_absmax;
  int e = 0;
  if (table_absmax > 0) frexp(table_absmax, &e);
  plan->mixed.a_exp = table_absmax > 0 ? e : 0;
  const int64_t n_elems =
      (int64_t)d.n_tables * d.n_cases * g.n_kc * kDigits * (int64_t)g.np * g.kc;
  plan->mixed.adig_elems = n_elems;
  build_adig_kernel<<<grid_for(n_elems, 256), 256, 0, s>>>(
      d, g, plan->mixed.adig, plan->mixed.a_exp);
  cudaError_t err = cudaGetLastError();
  return err == cudaSuccess ? VL1_OK : cuda_fail(err, "build_adig_kernel launch");
}

int64_t mixed_workspace_bytes(const vl1_plan *plan, int64_t nboxes, int64_t n_tgt_boxes,
                              int nrhs) {
  const MixedGeom &g = plan->mixed.geom;
  const int cv = plan->d.table_cplx ? 2 : 1;
  int64_t b = 0;
  b += ((int64_t)nrhs * 4 + 255) / 256 * 256;                       // rhs scale exponents
  b += (nboxes * nrhs * g.kp * kXPlanes * 2 + 255) / 256 * 256;    // density digit planes
  if (plan->d.disp_kind == VL1_DISP_LOG2D) {
    b += (nboxes * nrhs * cv * 8 + 255) / 256 * 256;            // per-box displacement
    b += (n_tgt_boxes * nrhs * cv * 8 + 255) / 256 * 256;       // per-target displacement
  }
  return b + 4096;
}

int32_t launch_classify(vl1_plan *plan, const TreeDev &tree, int32_t *keys, cudaStream_t s) {
  classify_pairs_kernel<<<grid_for(tree.n_tgt_boxes, 128), 128, 0, s>>>(plan->d, tree, keys,
                                                                         plan->status);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? VL1_OK : cuda_fail(e, "classify_pairs_kernel launch");
}

// Measurement hook (vl1_set_kernel_events): events recorded on the call's
// stream right before and after the tensor-core kernel launches.
cudaEvent_t g_kernel_begin = nullptr, g_kernel_end = nullptr;

// Test hook (vl1_test_set_wait_fault): time limit of the kernel's bounded
// waits in microseconds (0: the default) and the withheld arrival of CTA
// (0, 0).
uint32_t g_test_wait_limit_us = 0;
int32_t g_test_withhold = 0;

int32_t record_kernel_event(cudaEvent_t ev, cudaStream_t s) {
  if (!ev) return VL1_OK;
  cudaError_t e = cudaEventRecord(ev, s);
  return e == cudaSuccess ? VL1_OK : cuda_fail(e, "cudaEventRecord(kernel event)");
}

int32_t launch_mixed(vl1_plan *plan, const TreeDev &tree, int64_t nboxes,
                     const vl1_mixed_schedule &sched, const double *coefs, int nrhs,
                     double *result, void *workspace, int64_t ws_bytes, cudaStream_t s) {
  const DevDesc &d = plan->d;
  const MixedGeom &g = plan->mixed.geom;
  const int cv = d.table_cplx ? 2 : 1;
  const int64_t need = mixed_workspace_bytes(plan, nboxes, tree.n_tgt_boxes, nrhs);
  if (!workspace || ws_bytes < need) {
    set_error("mixed workspace of %lld bytes required, %lld given", (long long)need,
              (long long)ws_bytes);
    return VL1_E_ARG;
  }
  if (sched.n_splits > 0 && sched.n_chunks != g.np / g.nch) {
    set_error("the schedule's split scratch is for %d column chunks, the plan has %d",
              sched.n_chunks, g.np / g.nch);
    return VL1_E_ARG;
  }
  uint8_t *w = static_cast<uint8_t *>(workspace);
  const int64_t n_xrows = nboxes * nrhs;
  if (n_xrows >= INT32_MAX) {
    set_error("mixed path: %lld density rows exceed the 32-bit row index",
              (long long)n_xrows);
    return VL1_E_UNSUPPORTED;
  }
  int *x_exp = reinterpret_cast<int *>(w);
  w += ((int64_t)nrhs * 4 + 255) / 256 * 256;
  __half *xpl = reinterpret_cast<__half *>(w);
  w += (n_xrows * g.kp * kXPlanes * 2 + 255) / 256 * 256;
  double *wbox = nullptr, *disp = nullptr;
  if (d.disp_kind == VL1_DISP_LOG2D) {
    wbox = reinterpret_cast<double *>(w);
    w += (nboxes * nrhs * cv * 8 + 255) / 256 * 256;
    disp = reinterpret_cast<double *>(w);
  }
  cudaError_t e;
  const int64_t nbr = n_xrows;
  // the rhs scale exponents (maximum over all density rows), then the digit
  // planes of every density row
  e = cudaMemsetAsync(x_exp, 0, sizeof(int) * nrhs, s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(rhs exponents)");
  // a few blocks per SM, each warp striding over several rows: one global
  // atomic per block and rhs
  if (d.nq <= 32 && nrhs >= 4) {
    // small boxes, several rhs: a warp per (32 boxes, one rhs)
    const int64_t n_warp_tiles = (int64_t)((nboxes + 31) / 32) * nrhs;
    x_exponent_small_kernel<<<grid_for(n_warp_tiles * 32, 128), 128, 0, s>>>(
        d, tree, (int)nboxes, coefs, nrhs, x_exp);
  } else {
    // one warp per group of kRowGroup rows
    const int64_t n_groups = (nbr + kRowGroup - 1) / kRowGroup;
    x_exponent_kernel<<<grid_for(n_groups * 32, 256), 256, 0, s>>>(d, tree, (int)nboxes,
                                                                  coefs, nrhs, x_exp);
  }
  const size_t plane_smem = (size_t)4 * kPlaneGroup * g.kp * kXPlanes * 2;
  if (plane_smem > 48 * 1024) {
    e = cudaFuncSetAttribute(x_planes_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)plane_smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(x_planes_kernel)");
  }
  const int64_t n_plane_groups = (nbr + kPlaneGroup - 1) / kPlaneGroup;
  x_planes_kernel<<<grid_for(n_plane_groups * 32, 128), 128, plane_smem, s>>>(
      d, tree, (int)nboxes, coefs, nrhs, x_exp, xpl, g.kp, g.kc, plan->status);
  if (disp) {
    disp_box_kernel<<<grid_for(nbr, 256), 256, 0, s>>>(d, tree, (int)nboxes, coefs, nrhs,
                                                      wbox);
    disp_target_kernel<<<grid_for((int64_t)tree.n_tgt_boxes * nrhs, 256), 256, 0, s>>>(
        d, tree, nrhs, wbox, disp);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "mixed preparation launch");
  if (sched.n_tiles == 0) return VL1_OK;

  vl1::MixedParams mp;
  mp.d = d;
  mp.g = g;
  mp.nrhs = nrhs;
  mp.sched = sched;
  mp.xpl = xpl;
  mp.n_xrows = (int32_t)n_xrows;
  mp.adig = plan->mixed.adig;
  mp.x_exp = x_exp;
  mp.a_exp = plan->mixed.a_exp;
  mp.disp = disp;
  mp.target_boxes = tree.target_boxes;
  mp.tgt_starts = tree.tgt_starts;
  mp.tgt_counts = tree.tgt_counts;
  mp.n_tgt_boxes = tree.n_tgt_boxes;
  mp.n_particles = tree.n_particles;
  mp.result = result;
  mp.st = plan->status;
  mp.wait_limit_us = g_test_wait_limit_us;
  mp.withhold_arrival = g_test_withhold;
  if (!mixed_kernel_ptr(g.nch, g.kc, false)) {
    set_error("mixed path: unsupported column chunk %d / K chunk %d", g.nch, g.kc);
    return VL1_E_UNSUPPORTED;
  }
  dim3 grid(sched.n_items > 0 ? sched.n_items : sched.n_tiles, g.np / g.nch);
  BatchLaunch none{};
  int32_t st = record_kernel_event(g_kernel_begin, s);
  if (st) return st;
  e = launch_mixed_kernel(g.nch, g.kc, false, grid, s, mp, none);
  if (e != cudaSuccess) return cuda_fail(e, "mixed_kernel launch");
  return record_kernel_event(g_kernel_end, s);
}

}  // namespace vl1

// --------------------------------------------------------------- batches

namespace {

constexpr int kRowsPerTask = 64;

struct BatchGroup {   // problems sharing one kernel shape: one persistent launch
  int nch, kc;
  int item0, n_items;
  int grid;
};

// A problem large enough to fill the GPU on its own (two waves of CTAs or
// more): launched with one work item per CTA, its parameters by value (the
// persistent variant reads them from shared memory per item and is slower
// per item).
struct SoloLaunch {
  int problem;
  int nch, kc;
  int grid_x, grid_y;
  vl1::MixedParams mp;
};

int64_t round256(int64_t b) { return (b + 255) / 256 * 256; }

}  // namespace

struct vl1_batch {
  int device = -1;
  void *buf = nullptr;
  int64_t bytes = 0;
  int n_sm = 0;
  int ctas = 0;   // persistent CTAs per kernel shape (0: one per SM)
  int n_problems = 0;
  void *d_probs = nullptr, *d_prep = nullptr, *d_tasks = nullptr, *d_items = nullptr;
  int n_tasks = 0;
  int *d_queue = nullptr;
  void *d_ttasks = nullptr;   // target-row tasks of the 2D displacement sums
  int n_ttasks = 0;
  int *d_exp = nullptr;       // every problem's rhs scale exponents, contiguous
  int n_exp = 0;
  std::vector<BatchGroup> groups;
  std::vector<SoloLaunch> solos;
  bool has_disp = false;
  int max_row_bytes = 16;   // largest kp * 8 of the problems (digit plane staging)
  // pinned staging of vl1_batch_update (two, so that one can be refilled
  // while the copy from the other is in flight)
  void *pinned[2] = {nullptr, nullptr};
  int64_t pinned_bytes[2] = {0, 0};
  cudaEvent_t pinned_done[2] = {nullptr, nullptr};
  bool pinned_used[2] = {false, false};
  int flip = 0;
};

using namespace vl1;

namespace {

// Host assembly of one problem set: validated parameters, task and work
// lists, and the layout of the batch buffer ([parameters][workspaces]).
struct BatchLayout {
  std::vector<MixedParams> mps;
  std::vector<PrepProblem> preps;
  std::vector<int64_t> ws_need, nrows;
  std::vector<PrepTask> tasks, ttasks;
  std::vector<BatchItem> all;
  std::vector<BatchGroup> groups;
  std::vector<SoloLaunch> solos;
  int64_t o_probs = 0, o_prep = 0, o_tasks = 0, o_items = 0, o_queue = 0, o_ttasks = 0;
  int64_t o_exp = 0;          // the rhs scale exponents of all problems
  std::vector<int64_t> exp_off;   // a problem's first exponent in that region
  int64_t n_exp = 0;
  int64_t param_bytes = 0;   // the parameter region [0, param_bytes)
  std::vector<int64_t> o_ws;
  int64_t total_bytes = 0;
};

int32_t assemble_batch(const char *who, int dev, int n_sm, int ctas_opt, int32_t n_problems,
                       const vl1_batch_problem *problems, BatchLayout &L) {
  L = BatchLayout{};
  L.mps.resize(n_problems);
  L.preps.resize(n_problems);
  L.ws_need.resize(n_problems);
  L.nrows.resize(n_problems);
  std::vector<std::vector<vl1_mixed_item>> items(n_problems);
  cudaError_t e;
  for (int i = 0; i < n_problems; ++i) {
    const vl1_batch_problem &q = problems[i];
    if (!q.plan || !q.tree || !q.schedule || !q.coefs || !q.result || q.nrhs < 1) {
      set_error("%s: problem %d has a null plan/tree/schedule/coefs/result or nrhs < 1", who,
                i);
      return VL1_E_ARG;
    }
    if (q.plan->device != dev) {
      set_error("%s: problem %d's plan is on device %d, not the current %d", who, i,
                q.plan->device, dev);
      return VL1_E_ARG;
    }
    TreeDev tr;
    int32_t st = make_tree(q.plan, q.tree, tr);
    if (st) return st;
    const vl1_mixed_schedule &sc = *q.schedule;
    if (tr.nboxes < 1 || sc.n_tiles < 0 || sc.n_items < 0 ||
        (sc.n_tiles > 0 && (!sc.tile_rows || !sc.tile_key_start || !sc.key_ids ||
                            !sc.key_xrow)) ||
        (sc.n_items > 0 && !sc.items) ||
        reinterpret_cast<uintptr_t>(sc.key_xrow) % 16 != 0 ||
        (sc.n_splits > 0 && (!sc.split_counters || !sc.split_partials))) {
      set_error("%s: problem %d has an invalid tree or schedule", who, i);
      return VL1_E_ARG;
    }
    const MixedGeom &g = q.plan->mixed.geom;
    if (!mixed_kernel_ptr(g.nch, g.kc, true)) {
      set_error("%s: problem %d: unsupported kernel shape", who, i);
      return VL1_E_UNSUPPORTED;
    }
    if (sc.n_splits > 0 && sc.n_chunks != g.np / g.nch) {
      set_error("%s: problem %d: the schedule's split scratch is for %d column chunks, the "
                "plan has %d", who, i, sc.n_chunks, g.np / g.nch);
      return VL1_E_ARG;
    }
    L.nrows[i] = tr.nboxes * q.nrhs;
    if (L.nrows[i] >= INT32_MAX) {
      set_error("%s: problem %d has %lld density rows (32-bit row index)", who, i,
                (long long)L.nrows[i]);
      return VL1_E_UNSUPPORTED;
    }
    L.ws_need[i] = mixed_workspace_bytes(q.plan, tr.nboxes, tr.n_tgt_boxes, q.nrhs);
    MixedParams &mp = L.mps[i];
    mp = MixedParams{};
    mp.d = q.plan->d;
    mp.g = g;
    mp.nrhs = q.nrhs;
    mp.sched = sc;
    mp.n_xrows = (int32_t)L.nrows[i];
    mp.adig = q.plan->mixed.adig;
    mp.a_exp = q.plan->mixed.a_exp;
    mp.target_boxes = tr.target_boxes;
    mp.tgt_starts = tr.tgt_starts;
    mp.tgt_counts = tr.tgt_counts;
    mp.n_tgt_boxes = tr.n_tgt_boxes;
    mp.n_particles = tr.n_particles;
    mp.result = static_cast<double *>(q.result);
    mp.st = q.plan->status;
    PrepProblem &pp = L.preps[i];
    pp = PrepProblem{};
    pp.d = q.plan->d;
    pp.tr = tr;
    pp.coefs = q.coefs;
    pp.nrhs = q.nrhs;
    pp.kp = g.kp;
    pp.kc = g.kc;
    pp.st = q.plan->status;
    // the work list of this problem: the caller's host copy of the
    // schedule's items, else a copy from the device
    if (sc.n_items > 0 && q.host_items) {
      items[i].assign(q.host_items, q.host_items + sc.n_items);
    } else if (sc.n_items > 0) {
      items[i].resize(sc.n_items);
      e = cudaMemcpy(items[i].data(), sc.items, sizeof(vl1_mixed_item) * sc.n_items,
                     cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(schedule items)");
    } else if (sc.n_tiles > 0) {
      std::vector<int32_t> ks(sc.n_tiles + 1);
      e = cudaMemcpy(ks.data(), sc.tile_key_start, sizeof(int32_t) * ks.size(),
                     cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(tile_key_start)");
      for (int t = 0; t < sc.n_tiles; ++t)
        items[i].push_back(vl1_mixed_item{t, ks[t], ks[t + 1], -1, 0, 1, -1, 0});
    }
    for (const vl1_mixed_item &it : items[i]) {
      if (it.tile < 0 || it.tile >= sc.n_tiles || it.key_begin < 0 ||
          it.key_end < it.key_begin || it.nparts < 1 || it.part < 0 ||
          it.part >= it.nparts || it.nparts >= kSplitPoison || it.split >= sc.n_splits ||
          (it.split >= 0 && (it.slot < it.part || it.slot >= sc.n_slots))) {
        set_error("%s: problem %d has an invalid work item", who, i);
        return VL1_E_ARG;
      }
    }
  }
  // one program-wide check: two problems may not share split scratch
  for (int i = 0; i < n_problems; ++i)
    for (int j = i + 1; j < n_problems; ++j)
      if (problems[i].schedule->n_splits > 0 &&
          problems[i].schedule->split_counters == problems[j].schedule->split_counters) {
        set_error("%s: problems %d and %d share split scratch (one schedule per problem)",
                  who, i, j);
        return VL1_E_ARG;
      }

  // ---- combined work list: one group per kernel shape, longest items first
  struct Cand {
    int64_t cost;
    BatchItem it;
  };
  std::vector<char> solo(n_problems, 0);
  for (int i = 0; i < n_problems; ++i) {
    const vl1_mixed_schedule &sc = *problems[i].schedule;
    const MixedGeom &g = problems[i].plan->mixed.geom;
    const int64_t n_x = sc.n_items > 0 ? sc.n_items : sc.n_tiles;
    const int64_t ctas = n_x * (g.np / g.nch);
    if (ctas >= 2ll * n_sm * mixed_ctas_per_sm(g.nch) && n_x < INT32_MAX &&
        mixed_kernel_ptr(g.nch, g.kc, false)) {
      solo[i] = 1;
      SoloLaunch sl;
      sl.problem = i;
      sl.nch = g.nch;
      sl.kc = g.kc;
      sl.grid_x = (int)n_x;
      sl.grid_y = g.np / g.nch;
      L.solos.push_back(sl);
    }
  }
  std::vector<std::pair<int, int>> shapes;
  for (int i = 0; i < n_problems; ++i) {
    if (solo[i]) continue;
    const MixedGeom &g = problems[i].plan->mixed.geom;
    std::pair<int, int> sh(g.nch, g.kc);
    if (std::find(shapes.begin(), shapes.end(), sh) == shapes.end()) shapes.push_back(sh);
  }
  for (const auto &sh : shapes) {
    std::vector<Cand> cands;
    for (int i = 0; i < n_problems; ++i) {
      const MixedGeom &g = problems[i].plan->mixed.geom;
      if (solo[i] || g.nch != sh.first || g.kc != sh.second) continue;
      for (const vl1_mixed_item &it : items[i])
        for (int c = 0; c < g.np / g.nch; ++c)
          cands.push_back(Cand{(int64_t)(it.key_end - it.key_begin) * g.n_kc + 2,
                               BatchItem{i, c, it}});
    }
    std::stable_sort(cands.begin(), cands.end(),
                     [](const Cand &a, const Cand &b) { return a.cost > b.cost; });
    BatchGroup bg;
    bg.nch = sh.first;
    bg.kc = sh.second;
    bg.item0 = (int)L.all.size();
    bg.n_items = (int)cands.size();
    const int ctas = ctas_opt > 0 ? ctas_opt : n_sm * mixed_ctas_per_sm(sh.first);
    bg.grid = bg.n_items < ctas ? bg.n_items : ctas;
    for (const Cand &c : cands) L.all.push_back(c.it);
    if (bg.n_items > 0) L.groups.push_back(bg);
  }
  for (int i = 0; i < n_problems; ++i) {
    for (int64_t r0 = 0; r0 < L.nrows[i]; r0 += kRowsPerTask)
      L.tasks.push_back(
          PrepTask{i, (int32_t)std::min<int64_t>(kRowsPerTask, L.nrows[i] - r0), r0});
    const int64_t nt = (int64_t)L.preps[i].tr.n_tgt_boxes * problems[i].nrhs;
    for (int64_t r0 = 0; r0 < nt; r0 += 256)
      L.ttasks.push_back(PrepTask{i, (int32_t)std::min<int64_t>(256, nt - r0), r0});
  }

  // ---- layout: parameters, work list, queues, then the workspaces
  int64_t off = 0;
  L.o_probs = off;
  off += round256(sizeof(MixedParams) * n_problems);
  L.o_prep = off;
  off += round256(sizeof(PrepProblem) * n_problems);
  L.o_tasks = off;
  off += round256(sizeof(PrepTask) * (L.tasks.size() + 1));
  L.o_items = off;
  off += round256(sizeof(BatchItem) * (L.all.size() + 1));
  L.o_queue = off;
  off += round256(sizeof(int) * (L.groups.size() + 1));
  L.o_ttasks = off;
  off += round256(sizeof(PrepTask) * (L.ttasks.size() + 1));
  L.param_bytes = off;
  L.exp_off.resize(n_problems);
  L.n_exp = 0;
  for (int i = 0; i < n_problems; ++i) {
    L.exp_off[i] = L.n_exp;
    L.n_exp += problems[i].nrhs;
  }
  L.o_exp = off;
  off += round256(sizeof(int) * L.n_exp);
  L.o_ws.resize(n_problems);
  for (int i = 0; i < n_problems; ++i) {
    L.o_ws[i] = off;
    off += round256(L.ws_need[i]);
  }
  L.total_bytes = off;
  return VL1_OK;
}

// Point every problem at its workspace inside the buffer at `base` and make
// the batch's launch lists; `host` receives the parameter region's bytes.
void place_batch(vl1_batch *b, BatchLayout &L, const vl1_batch_problem *problems,
                 std::vector<uint8_t> *host, uint8_t *host_ptr) {
  uint8_t *base = static_cast<uint8_t *>(b->buf);
  const int n_problems = (int)L.mps.size();
  b->has_disp = false;
  b->max_row_bytes = 16;
  for (int i = 0; i < n_problems; ++i) {
    const vl1_batch_problem &q = problems[i];
    const MixedGeom &g = q.plan->mixed.geom;
    const int cv = q.plan->d.table_cplx ? 2 : 1;
    uint8_t *w = base + L.o_ws[i];
    // a problem's workspace: [digit planes][disp] (its rhs exponents are
    // in the batch's exponent region, cleared by one memset per evaluation)
    int *x_exp = reinterpret_cast<int *>(base + L.o_exp) + L.exp_off[i];
    __half *xpl = reinterpret_cast<__half *>(w);
    w += round256(L.nrows[i] * g.kp * kXPlanes * 2);
    double *wbox = nullptr, *disp = nullptr;
    if (q.plan->d.disp_kind == VL1_DISP_LOG2D) {
      wbox = reinterpret_cast<double *>(w);
      w += round256(L.nrows[i] * cv * 8);
      disp = reinterpret_cast<double *>(w);
      b->has_disp = true;
    }
    L.mps[i].xpl = xpl;
    L.mps[i].x_exp = x_exp;
    L.mps[i].disp = disp;
    L.preps[i].x_exp = x_exp;
    L.preps[i].xpl = xpl;
    b->max_row_bytes = std::max(b->max_row_bytes, g.kp * kXPlanes * 2);
    L.preps[i].wbox = wbox;
    L.preps[i].disp = disp;
  }
  b->solos = L.solos;
  for (SoloLaunch &sl : b->solos) sl.mp = L.mps[sl.problem];
  b->n_problems = n_problems;
  b->d_probs = base + L.o_probs;
  b->d_prep = base + L.o_prep;
  b->d_tasks = base + L.o_tasks;
  b->d_items = base + L.o_items;
  b->n_tasks = (int)L.tasks.size();
  b->d_queue = reinterpret_cast<int *>(base + L.o_queue);
  b->d_ttasks = base + L.o_ttasks;
  b->n_ttasks = (int)L.ttasks.size();
  b->d_exp = reinterpret_cast<int *>(base + L.o_exp);
  b->n_exp = (int)L.n_exp;
  b->groups = L.groups;
  uint8_t *h = host_ptr;
  if (host) {
    host->assign(L.param_bytes, 0);
    h = host->data();
  }
  auto put = [&](int64_t o, const void *src, size_t n) {
    if (n) std::memcpy(h + o, src, n);
  };
  put(L.o_probs, L.mps.data(), sizeof(MixedParams) * L.mps.size());
  put(L.o_prep, L.preps.data(), sizeof(PrepProblem) * L.preps.size());
  put(L.o_tasks, L.tasks.data(), sizeof(PrepTask) * L.tasks.size());
  put(L.o_items, L.all.data(), sizeof(BatchItem) * L.all.size());
  put(L.o_ttasks, L.ttasks.data(), sizeof(PrepTask) * L.ttasks.size());
}

int32_t set_batch_smem(const std::vector<BatchGroup> &groups,
                       const std::vector<SoloLaunch> &solos) {
  for (const BatchGroup &g : groups) {
    cudaError_t e = cudaFuncSetAttribute(mixed_kernel_ptr(g.nch, g.kc, true),
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)mixed_smem_bytes(g.nch, g.kc));
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(batch kernel)");
  }
  for (const SoloLaunch &sl : solos) {
    cudaError_t e = cudaFuncSetAttribute(mixed_kernel_ptr(sl.nch, sl.kc, false),
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)mixed_smem_bytes(sl.nch, sl.kc));
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(batch kernel)");
  }
  return VL1_OK;
}

}  // namespace

extern "C" int32_t vl1_batch_create(int32_t n_problems, const vl1_batch_problem *problems,
                                    const vl1_batch_options *options, vl1_batch **out) {
  if (!out || n_problems < 1 || !problems) {
    set_error("vl1_batch_create: no problems or null output");
    return VL1_E_ARG;
  }
  *out = nullptr;
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  int n_sm = 0;
  e = cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
  const int ctas = options && options->ctas_per_launch > 0 ? options->ctas_per_launch : 0;
  const int64_t capacity = options && options->capacity_bytes > 0 ? options->capacity_bytes : 0;
  BatchLayout L;
  int32_t st = assemble_batch("vl1_batch_create", dev, n_sm, ctas, n_problems, problems, L);
  if (st) return st;
  vl1_batch *b = new vl1_batch();
  b->device = dev;
  b->n_sm = n_sm;
  b->ctas = ctas;
  b->bytes = std::max(L.total_bytes, capacity);
  e = cudaMalloc(&b->buf, b->bytes);
  if (e != cudaSuccess) {
    delete b;
    return cuda_fail(e, "cudaMalloc(batch)");
  }
  std::vector<uint8_t> host;
  place_batch(b, L, problems, &host, nullptr);
  e = cudaMemcpy(b->buf, host.data(), host.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(b->buf);
    delete b;
    return cuda_fail(e, "cudaMemcpy(batch parameters)");
  }
  st = set_batch_smem(b->groups, b->solos);
  if (st) {
    cudaFree(b->buf);
    delete b;
    return st;
  }
  *out = b;
  return VL1_OK;
}

extern "C" int32_t vl1_batch_update(vl1_batch *b, int32_t n_problems,
                                    const vl1_batch_problem *problems, void *stream) {
  if (!b || n_problems < 1 || !problems) {
    set_error("vl1_batch_update: null batch or no problems");
    return VL1_E_ARG;
  }
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev != b->device) {
    set_error("vl1_batch_update: batch is on device %d, not the current %d", b->device, dev);
    return VL1_E_ARG;
  }
  BatchLayout L;
  int32_t st = assemble_batch("vl1_batch_update", dev, b->n_sm, b->ctas, n_problems, problems, L);
  if (st) return st;
  if (L.total_bytes > b->bytes) {
    set_error("vl1_batch_update: the problems need %lld bytes, the batch holds %lld",
              (long long)L.total_bytes, (long long)b->bytes);
    return VL1_E_ARG;
  }
  // refill the staging buffer whose last copy is oldest
  const int k = b->flip;
  b->flip ^= 1;
  if (b->pinned_used[k]) {
    e = cudaEventSynchronize(b->pinned_done[k]);
    if (e != cudaSuccess) return cuda_fail(e, "cudaEventSynchronize(batch staging)");
  }
  if (!b->pinned_done[k]) {
    e = cudaEventCreateWithFlags(&b->pinned_done[k], cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(e, "cudaEventCreate(batch staging)");
  }
  if (b->pinned_bytes[k] < L.param_bytes) {
    if (b->pinned[k]) cudaFreeHost(b->pinned[k]);
    b->pinned[k] = nullptr;
    b->pinned_bytes[k] = 0;
    const int64_t want = std::max<int64_t>(L.param_bytes * 2, 1 << 16);
    e = cudaMallocHost(&b->pinned[k], want);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMallocHost(batch staging)");
    b->pinned_bytes[k] = want;
  }
  place_batch(b, L, problems, nullptr, static_cast<uint8_t *>(b->pinned[k]));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  e = cudaMemcpyAsync(b->buf, b->pinned[k], L.param_bytes, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(batch parameters)");
  e = cudaEventRecord(b->pinned_done[k], s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaEventRecord(batch staging)");
  b->pinned_used[k] = true;
  return set_batch_smem(b->groups, b->solos);
}

extern "C" int32_t vl1_batch_eval(vl1_batch *b, void *stream) {
  if (!b) {
    set_error("vl1_batch_eval: null batch");
    return VL1_E_ARG;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(b->d_queue, 0, sizeof(int) * b->groups.size(), s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(batch)");
  if (b->n_exp > 0) {
    e = cudaMemsetAsync(b->d_exp, 0, sizeof(int) * b->n_exp, s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(batch exponents)");
  }
  if (b->n_tasks > 0) {
    x_exponent_batch_kernel<<<b->n_tasks, 256, 0, s>>>(
        static_cast<const PrepProblem *>(b->d_prep), static_cast<const PrepTask *>(b->d_tasks));
    const size_t plane_smem = (size_t)4 * kPlaneGroup * b->max_row_bytes;
    if (plane_smem > 48 * 1024) {
      e = cudaFuncSetAttribute(x_planes_batch_kernel,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)plane_smem);
      if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(x_planes_batch_kernel)");
    }
    x_planes_batch_kernel<<<b->n_tasks, 128, plane_smem, s>>>(
        static_cast<const PrepProblem *>(b->d_prep), static_cast<const PrepTask *>(b->d_tasks),
        b->max_row_bytes);
  }
  if (b->has_disp && b->n_tasks > 0) {
    disp_box_batch_kernel<<<b->n_tasks, 64, 0, s>>>(static_cast<const PrepProblem *>(b->d_prep),
                                                    static_cast<const PrepTask *>(b->d_tasks));
    if (b->n_ttasks > 0)
      disp_target_batch_kernel<<<b->n_ttasks, 256, 0, s>>>(
          static_cast<const PrepProblem *>(b->d_prep),
          static_cast<const PrepTask *>(b->d_ttasks));
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "batch preparation launch");
  const MixedParams unused{};
  int32_t st = record_kernel_event(g_kernel_begin, s);
  if (st) return st;
  for (const SoloLaunch &sl : b->solos) {
    const BatchLaunch none{};
    MixedParams mp = sl.mp;
    mp.wait_limit_us = g_test_wait_limit_us;
    mp.withhold_arrival = g_test_withhold;
    void *args[] = {&mp, const_cast<BatchLaunch *>(&none)};
    e = cudaLaunchKernel(mixed_kernel_ptr(sl.nch, sl.kc, false), dim3(sl.grid_x, sl.grid_y),
                         dim3(mixed_threads(sl.nch)), args, mixed_smem_bytes(sl.nch, sl.kc), s);
    if (e != cudaSuccess) return cuda_fail(e, "batch mixed_kernel launch (one problem)");
  }
  for (size_t gi = 0; gi < b->groups.size(); ++gi) {
    const BatchGroup &g = b->groups[gi];
    BatchLaunch bl;
    bl.probs = static_cast<const MixedParams *>(b->d_probs);
    bl.items = static_cast<const BatchItem *>(b->d_items) + g.item0;
    bl.n_items = g.n_items;
    bl.queue = b->d_queue + gi;
    bl.wait_limit_us = g_test_wait_limit_us;
    bl.withhold_arrival = g_test_withhold;
    void *args[] = {const_cast<MixedParams *>(&unused), &bl};
    e = cudaLaunchKernel(mixed_kernel_ptr(g.nch, g.kc, true), dim3(g.grid),
                         dim3(mixed_threads(g.nch)), args, mixed_smem_bytes(g.nch, g.kc), s);
    if (e != cudaSuccess) return cuda_fail(e, "batch mixed_kernel launch");
  }
  return record_kernel_event(g_kernel_end, s);
}

extern "C" int32_t vl1_batch_destroy(vl1_batch *b) {
  if (!b) return VL1_OK;
  for (int k = 0; k < 2; ++k) {
    if (b->pinned_used[k]) cudaEventSynchronize(b->pinned_done[k]);
    if (b->pinned_done[k]) cudaEventDestroy(b->pinned_done[k]);
    if (b->pinned[k]) cudaFreeHost(b->pinned[k]);
  }
  cudaError_t e = b->buf ? cudaFree(b->buf) : cudaSuccess;
  delete b;
  return e == cudaSuccess ? VL1_OK : cuda_fail(e, "cudaFree(batch)");
}

extern "C" int64_t vl1_batch_device_bytes(const vl1_batch *b) { return b ? b->bytes : -1; }

extern "C" int32_t vl1_batch_kernel_launches(const vl1_batch *b) {
  if (!b) return -1;
  int n = 0;
  if (b->n_tasks > 0) n += 2;   // exponents, digit planes
  if (b->has_disp && b->n_tasks > 0) n += 1 + (b->n_ttasks > 0 ? 1 : 0);
  return n + (int)b->solos.size() + (int)b->groups.size();
}

extern "C" int32_t vl1_test_set_wait_fault(int32_t wait_limit_us, int32_t withhold_arrival) {
  if (wait_limit_us < 0) {
    set_error("vl1_test_set_wait_fault: negative wait limit");
    return VL1_E_ARG;
  }
  vl1::g_test_wait_limit_us = (uint32_t)wait_limit_us;
  vl1::g_test_withhold = withhold_arrival != 0;
  return VL1_OK;
}

extern "C" int32_t vl1_set_kernel_events(void *begin, void *end) {
  vl1::g_kernel_begin = static_cast<cudaEvent_t>(begin);
  vl1::g_kernel_end = static_cast<cudaEvent_t>(end);
  return VL1_OK;
}
