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
// call) are written in fixed point against per-plan / per-row power-of-two
// scales, both as 39-bit magnitudes: the table in balanced base-256 digits
// (|digit| <= 128, times the value's sign), the densities as a 7-bit top
// digit and four base-256 digits carrying the value's sign (|digit| <= 127
// for the top one, <= 255 for the others), all held exactly in FP16.
// Densities are stored as bytes (sign in bit 7 of the top digit) and expanded
// to FP16 in shared memory.  A diagonal i + j of digit products summed over
// K <= 64 source points is an integer below 2^22 for i + j <= 3 and below
// 2^24 for i + j = 4, exact in the FP32 accumulator.  Those diagonals (the
// leading 32 bits) get their own TMEM accumulator, re-initialised per K round
// and read after every round into int64 registers: one FADD with 1.5 * 2^23
// turns an exact d <= 3 float into its integer bits, d = 4 takes a
// conversion; diagonals i + j = 5, 6 accumulate across rounds in FP32 TMEM
// (their rounding is below 2^-40 of the result); the products i + j >= 7 are
// dropped, and with balanced table digits they are zero-mean.  Each output's
// sum is then one exact integer, rounded once to FP64.
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
  if (M == 0) {
    m = 0;
  } else if (sh >= 0) {
    // saturates when |v| is not below 2^e (m >= 2^BITS after the shift)
    m = (sh > BITS || M >= (1ull << (BITS - sh))) ? (1ull << BITS) : (M << sh);
  } else if (sh < -63) {
    m = 0;
  } else {
    const int k = (int)-sh;
    const unsigned long long q = M >> k;
    const unsigned long long rem = M & ((1ull << k) - 1ull);
    const unsigned long long half = 1ull << (k - 1);
    m = q + ((rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull);
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
  long long r = (long long)fixed_magnitude<kFixedBits>(v, e);
  const int sgn = __double_as_longlong(v) < 0 ? -1 : 1;
#pragma unroll
  for (int i = kDigits - 1; i >= 1; --i) {
    int lo = (int)(r & 0xFF);
    lo -= lo >= 128 ? 256 : 0;
    dig[i] = sgn * lo;
    r = (r - lo) >> kDigitBits;
  }
  dig[0] = sgn * (int)r;   // m < 2^39: r <= 128
}

// density digit bytes: v = sign * 2^(e - 39) * m, m < 2^39; byte 0 holds
// the sign (bit 7) and the top 7 bits of m, bytes 1..4 the following
// base-256 digits of m (magnitudes)
__device__ __forceinline__ void density_digit_bytes(double v, int e, uint8_t (&byt)[kDigits]) {
  const unsigned long long m = fixed_magnitude<kXFixedBits>(v, e);
  const unsigned sgn = __double_as_longlong(v) < 0 ? 0x80u : 0u;
  byt[0] = (uint8_t)(sgn | (unsigned)((m >> (kXFixedBits - 7)) & 0x7F));
#pragma unroll
  for (int i = 1; i < kDigits; ++i)
    byt[i] = (uint8_t)((m >> (kXFixedBits - 7 - kDigitBits * i)) & 0xFF);
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

// one problem of a batch, as the preparation kernels see it
struct PrepProblem {
  DevDesc d;
  TreeDev tr;
  const double *coefs;
  int nrhs;
  int *x_exp;     // per density row
  int *ref_exp;   // per target row (target box index * nrhs + rhs)
  uint8_t *xdig;
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

// warp-wide maximum exponent of scaling * coefficient over row idx = b * nrhs
// + r (-1074 for an empty row); the same value in every lane
__device__ __forceinline__ int row_exponent(const DevDesc &d, const TreeDev &tr,
                                            const double *coefs, int nrhs, int64_t idx,
                                            int lane) {
  const int b = (int)(idx / nrhs), r = (int)(idx % nrhs);
  const int cnt = min(tr.src_counts[b], d.nq);
  int e = -1074;
  if (cnt > 0) {
    const double sc = box_scaling(d, tr, tr.levels[b]);
    const double *c = coefs + (int64_t)r * tr.n_particles + tr.src_starts[b];
    for (int s = lane; s < cnt; s += 32) e = max(e, scale_exponent(sc * c[s]));
  }
  return __reduce_max_sync(0xffffffffu, e);
}

// x digits: row R = b * nrhs + r holds [K chunk][digit][kc] bytes (kp * 5),
// so that the digits of one pipeline unit are one contiguous 5 * kc-byte
// piece at byte kchunk * 5 * kc; source points sit at their mode id.  One
// warp per row: the row's exponent (written to x_exp), then its digit bytes
// assembled in the warp's shared-memory slice `stage` (row_bytes, 16-byte
// aligned) and written out with 16-byte stores.
__device__ __forceinline__ void row_digits(const DevDesc &d, const TreeDev &tr,
                                           const double *coefs, int nrhs, int *x_exp,
                                           uint8_t *xdig, int kp, int kc, vl1_status *st,
                                           int64_t idx, int lane, uint8_t *stage) {
  const int row_bytes = kp * kDigits;
  const int b = (int)(idx / nrhs), r = (int)(idx % nrhs);
  int cnt = tr.src_counts[b];
  const int s0 = tr.src_starts[b];
  const int lev = tr.levels[b];
  if (cnt > d.nq) {
    if (lane == 0) report(st, VL1_E_LAYOUT, b, cnt);
    cnt = d.nq;
  }
  for (int k = lane * 16; k < row_bytes; k += 32 * 16)
    *reinterpret_cast<uint4 *>(stage + k) = make_uint4(0u, 0u, 0u, 0u);
  if (cnt > 0 && cnt <= 64) {
    // one pass (up to two values per lane): the scaled values, their mode
    // ids and the row exponent are loaded / formed once
    const double sc = box_scaling(d, tr, lev);
    const double *c = coefs + (int64_t)r * tr.n_particles + s0;
    const bool h0 = lane < cnt, h1 = lane + 32 < cnt;
    const double v0 = h0 ? sc * c[lane] : 0.0, v1 = h1 ? sc * c[lane + 32] : 0.0;
    const int m0 = h0 ? tr.smode[s0 + lane] : 0, m1 = h1 ? tr.smode[s0 + lane + 32] : 0;
    int e = max(h0 ? scale_exponent(v0) : -1074, h1 ? scale_exponent(v1) : -1074);
    e = __reduce_max_sync(0xffffffffu, e);
    if (lane == 0) x_exp[idx] = e;
    __syncwarp();
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const bool have = h ? h1 : h0;
      const int m = h ? m1 : m0;
      if (!have) continue;
      if (m < 0 || m >= d.nq) {
        report(st, VL1_E_LAYOUT, b, -1 - (lane + 32 * h));
        continue;
      }
      uint8_t byt[kDigits];
      density_digit_bytes(h ? v1 : v0, e, byt);
      const int base = (m / kc) * kDigits * kc + (m % kc);
#pragma unroll
      for (int i = 0; i < kDigits; ++i) stage[base + i * kc] = byt[i];
    }
  } else {
    const int e = row_exponent(d, tr, coefs, nrhs, idx, lane);
    if (lane == 0) x_exp[idx] = e;
    __syncwarp();
    if (cnt > 0) {
      const double sc = box_scaling(d, tr, lev);
      const double *c = coefs + (int64_t)r * tr.n_particles + s0;
      for (int s = lane; s < cnt; s += 32) {
        const int m = tr.smode[s0 + s];
        if (m < 0 || m >= d.nq) {
          report(st, VL1_E_LAYOUT, b, -1 - s);
          continue;
        }
        uint8_t byt[kDigits];
        density_digit_bytes(sc * c[s], e, byt);
        const int base = (m / kc) * kDigits * kc + (m % kc);
#pragma unroll
        for (int i = 0; i < kDigits; ++i) stage[base + i * kc] = byt[i];
      }
    }
  }
  __syncwarp();
  uint8_t *row = xdig + idx * row_bytes;
  for (int k = lane * 16; k < row_bytes; k += 32 * 16)
    *reinterpret_cast<uint4 *>(row + k) = *reinterpret_cast<const uint4 *>(stage + k);
  __syncwarp();
}

// Scale exponents.  Every density row (source box, rhs) gets its own: the
// exponent e with |scaling * coefficient| < 2^e over the box (-1074 for an
// empty or zero row); its digits are fixed point against 2^e.  Every target
// row (target box, rhs) gets the largest exponent of its list-1 source rows:
// its sum is accumulated in units of that exponent, so the precision of an
// output is relative to its own largest contribution.
__device__ __forceinline__ int target_row_exponent(const TreeDev &tr, int nrhs,
                                                   const int *x_exp, int64_t idx) {
  const int tb = (int)(idx / nrhs), r = (int)(idx % nrhs);
  int e = -1074;
  for (int p = tr.starts[tb]; p < tr.starts[tb + 1]; ++p)
    e = max(e, x_exp[(int64_t)tr.lists[p] * nrhs + r]);
  return e;
}

__global__ void ref_exponent_kernel(TreeDev tr, int nrhs, const int *x_exp, int *ref_exp) {
  const int64_t n = (int64_t)tr.n_tgt_boxes * nrhs;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x)
    ref_exp[idx] = target_row_exponent(tr, nrhs, x_exp, idx);
}

// dynamic shared memory: (blockDim.x / 32) x kp * 5 bytes (kp <= 1024 modes,
// a multiple of 16, so every warp's slice and row stays 16-byte aligned)
// (five blocks of 256 per SM: 46 registers, no spills)
__global__ void __launch_bounds__(256, 5)
    x_digits_kernel(DevDesc d, TreeDev tr, int nboxes, const double *coefs, int nrhs,
                    int *x_exp, uint8_t *xdig, int kp, int kc, vl1_status *st) {
  extern __shared__ __align__(16) uint8_t s_stage[];
  const int64_t n = (int64_t)nboxes * nrhs;
  const int lane = threadIdx.x & 31;
  uint8_t *stage = s_stage + (threadIdx.x >> 5) * kp * kDigits;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t idx = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; idx < n;
       idx += warps)
    row_digits(d, tr, coefs, nrhs, x_exp, xdig, kp, kc, st, idx, lane, stage);
}

// Batch versions: block i handles rows [row0, row0 + nrows) of one problem
// (tasks built on the host).  Target rows: one thread each.
__global__ void ref_exponent_batch_kernel(const PrepProblem *probs, const PrepTask *tasks) {
  const PrepTask t = tasks[blockIdx.x];
  const PrepProblem &P = probs[t.problem];
  for (int i = threadIdx.x; i < t.nrows; i += blockDim.x)
    P.ref_exp[t.row0 + i] = target_row_exponent(P.tr, P.nrhs, P.x_exp, t.row0 + i);
}

// Density rows: 8 warps striding over them.  Dynamic shared memory:
// (blockDim.x / 32) x (largest kp) * 5 bytes, at most 8 x 1024 x 5 = 40 KB.
__global__ void x_digits_batch_kernel(const PrepProblem *probs, const PrepTask *tasks,
                                      int max_row_bytes) {
  extern __shared__ __align__(16) uint8_t s_stage[];
  const PrepTask t = tasks[blockIdx.x];
  const PrepProblem &P = probs[t.problem];
  const int lane = threadIdx.x & 31;
  uint8_t *stage = s_stage + (threadIdx.x >> 5) * max_row_bytes;
  for (int64_t i = threadIdx.x >> 5; i < t.nrows; i += blockDim.x >> 5)
    row_digits(P.d, P.tr, P.coefs, P.nrhs, P.x_exp, P.xdig, P.kp, P.kc, P.st, t.row0 + i,
               lane, stage);
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

// round(x * 2^s) to the nearest int64 (ties to even) with integer operations
// (64-bit conversions run on the narrow FP64 side of this GPU); |x| * 2^s
// must stay below 2^62, which the FP32 tail accumulators do by far
__device__ __forceinline__ long long f32_scaled_to_i64(float x, int s) {
  const uint32_t b = __float_as_uint(x);
  const int e = (int)((b >> 23) & 0xFFu);
  if (e == 0) return 0;   // zero or subnormal: rounds to 0
  const long long m = (long long)((b & 0x7FFFFFu) | 0x800000u);
  const int sh = e - 150 + s;   // |x| * 2^s = m * 2^sh
  long long q;
  if (sh >= 0) {
    q = m << sh;
  } else if (sh < -25) {
    q = 0;                      // below 1/4
  } else {
    const int k = -sh;
    q = m >> k;
    const long long rem = m & ((1ll << k) - 1);
    const long long half = 1ll << (k - 1);
    q += (rem > half || (rem == half && (q & 1))) ? 1 : 0;
  }
  return (b >> 31) ? -q : q;
}

// ---------------------------------------------------------- main kernel

struct MixedParams {
  DevDesc d;
  MixedGeom g;
  int nrhs;
  vl1_mixed_schedule sched;
  const uint8_t *xdig;   // density digit bytes [n_xrows][kp * 5]
  int32_t n_xrows;
  const __half *adig;
  const int *x_exp;     // per density row
  const int *ref_exp;   // per target row
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
//   w <  8      producers: per pipeline unit, warp w gathers the density digit
//               bytes of tile rows 16w .. 16w+15 with cp.async (consecutive
//               lanes on consecutive 16-byte pieces of a row's 5 * kc bytes,
//               zero-filled for rows without a source box) into a staging
//               ring, then expands them to FP16 digit planes in the stage and
//               arrives on full[stage].  Eight warps keep enough requests in
//               flight to cover the L2 latency of these scattered rows.
//   w == 8      table loader (one lane): the five table digit tiles of the
//               unit's key by bulk copies (TMA), counted on full[stage]
//   w == 9      tensor-core issuer (one lane)
//   w >= 10     readout: TMEM lane quadrant w % 4, RC columns each
// Pipeline unit = (key, K chunk of kc <= 32 source points); a "round" = the
// units of one key that share an exact accumulation (K <= 64).  Exact
// diagonal accumulators (i+j = 2, 3, 4) are double-buffered in TMEM (one
// buffer per round parity) so the readout of round r overlaps the products of
// round r+1; the tail diagonals (i+j = 5, 6) accumulate over the whole tile.
// The table digit planes j = 1..5 of a stage are stacked along N, so one MMA
// multiplies density digit i by several table digits j at once; its output
// column blocks land on consecutive diagonals i + j.
// Density planes of a stage: the exact digits X1, X2, X3 and, for the tails
// only, R = X4 + X5 / 256 rounded to FP16 (11 significant bits: the density
// keeps ~2^-35 of its row's reference scale in the tails, far below the
// 2^-24 weight of the tails; the exact diagonals use X1..X3 only).
constexpr int kStages = 3;
constexpr int kXPlanes = 4;          // density planes per stage: X1, X2, X3, R
constexpr int kStgDepth = 3;         // byte staging ring per producer warp
constexpr uint32_t kExactCols = 3;   // accumulators per buffer
constexpr int kProducerWarps = 8;
constexpr int kRowsPerProducer = 128 / kProducerWarps;
constexpr int kLoaderWarp = 8;
constexpr int kMmaWarp = 9;
constexpr int kReadWarp0 = 10;
constexpr uint32_t kSleepNs = 200000;      // suspend hint of one barrier test
constexpr uint32_t kWaitLimitUs = 2000000; // a wait gives up after 2 s
// split-tile counters: parts in the low 16 bits, aborted parts also in the
// high bits (a tile has fewer than 2^16 parts)
constexpr int kSplitPoison = 1 << 16;

struct Barriers {
  uint64_t xfull[kStages];   // the producer warps' density planes are in the stage
  uint64_t afull[kStages];   // the table digit tiles have landed
  uint64_t empty[kStages];
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
__global__ void __launch_bounds__(32 * (kReadWarp0 + 4 * (NCH / 16)), 1)
mixed_kernel(const __grid_constant__ MixedParams p1, const __grid_constant__ BatchLaunch bl) {
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
      tc::mbar_init(&bars.xfull[s], kProducerWarps);   // one arrival per producer warp
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
  const int upr = (p.g.kp < 64 ? p.g.kp : 64) / KC;   // units per round
  const int rpk = (p.g.kp + 63) / 64;                  // rounds per key
  const int n_rounds = n_keys * rpk;

  if (tid < 128) {
    int v = p.sched.tile_rows[(int64_t)tile * 128 + tid];
    if (v >= (int64_t)p.n_tgt_boxes * p.nrhs) {
      report(p.st, VL1_E_ARG, tile, tid);
      v = -1;
    }
    s_rows[tid] = v;
  }
  __syncthreads();

  if (warp < kProducerWarps) {
    // ------------------------------------------------------------ producers
    // Per unit: gather the byte digits of this warp's 16 rows (5 * KC bytes
    // per row, cp.async into a kStgDepth-deep staging ring), then, kStgDepth
    // - 1 units behind, expand that unit's bytes to FP16 digit planes in the
    // unit's pipeline stage.  (One bulk copy per row instead was measured
    // slower: the copies queue behind each other in the copy engine.)
    constexpr int RB = kDigits * KC;           // bytes per row and unit
    constexpr int PPR = RB / 16;               // 16-byte pieces per row and unit
    constexpr int NH = KC / 16;                // 16-value halves per digit row
    constexpr int LOOK = kStgDepth - 1;        // units gathered ahead of the expansion
    const int64_t row_bytes = (int64_t)p.g.kp * kDigits;
    uint8_t *stg = smem + (size_t)kStages * STAGE_BYTES +
                   (size_t)warp * kStgDepth * kRowsPerProducer * RB;
    // lanes < kRowsPerProducer hold the source row of tile row my_row and
    // the reference exponent of its target row
    const int my_row = kRowsPerProducer * warp + (lane % kRowsPerProducer);
    int my_ref = 0;
    {
      const int v = s_rows[my_row];
      if (v >= 0) my_ref = p.ref_exp[v];
    }
    // key id, this lane's source row and its exponent, fetched one key
    // ahead; the source row two keys ahead, so that the exponent load never
    // waits for the row load
    int nkey = 0, nxr = -1, nxe = 0, nnxr = -1;
    if (n_keys > 0) {
      nkey = p.sched.key_ids[k0];
      nxr = p.sched.key_xrow[(int64_t)k0 * 128 + my_row];
      if (nxr >= 0 && nxr < p.n_xrows) nxe = p.x_exp[nxr];
    }
    if (n_keys > 1) nnxr = p.sched.key_xrow[(int64_t)(k0 + 1) * 128 + my_row];
    // right shift of the staged digits of units with even / odd index: a
    // source row's digits are fixed point against its own exponent and are
    // moved to the target row's reference exponent as they are expanded
    static_assert(kStgDepth == 3, "one shift register per staging slot");
    int sh_s0 = 0, sh_s1 = 0, sh_s2 = 0;
    // bit (u % kStgDepth): none of this warp's rows has a source box in unit
    // u (nothing gathered, zero planes); bit s of zero_stages: this warp's
    // rows of stage s hold zero planes (the stages are overwritten by the
    // parked sums at the end of an item, so the bits start clear per item)
    uint32_t empty_bits = 0, zero_stages = 0;
    // expand the staged bytes of unit v into stage v % kStages
    auto expand = [&](int v) -> bool {
      const int s = (ubase + v) % kStages;
      const int use = (ubase + v) / kStages;
      if (use > 0 && !wait_or_abort(&bars.empty[s], (use - 1) & 1, &s_abort, limit_us, true))
        return false;
      const uint8_t *sb = stg + (v % kStgDepth) * kRowsPerProducer * RB;
      uint8_t *xs = smem + (size_t)s * STAGE_BYTES;
      if ((empty_bits >> (v % kStgDepth)) & 1u) {
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
        if (lane == 0 && !(withhold && warp == 0 && ubase + v == 0))
          mbar_arrive(&bars.xfull[s]);
        return true;
      }
      zero_stages &= ~(1u << s);
      const __half2 k1024 = __floats2half2_rn(1024.0f, 1024.0f);
      constexpr int ITER = (kRowsPerProducer * NH + 31) / 32;
      const int vs = v % kStgDepth;
      const int shv = vs == 0 ? sh_s0 : (vs == 1 ? sh_s1 : sh_s2);
      int shr[ITER];
#pragma unroll
      for (int i = 0; i < ITER; ++i)
        shr[i] = __shfl_sync(0xffffffffu, shv, min((lane + 32 * i) / NH, kRowsPerProducer - 1));
#pragma unroll
      for (int i = 0; i < ITER; ++i) {
        const int t = lane + 32 * i;
        if (t >= kRowsPerProducer * NH) break;
        const int rl = t / NH, h = t - (t / NH) * NH;
        const uint8_t *src = sb + rl * RB + h * 16;
        // sign masks of the FP16 pairs (values 4q + 0/1 and 4q + 2/3): the
        // sign of a value is bit 7 of its top digit byte
        const uint4 top = *reinterpret_cast<const uint4 *>(src);
        const uint32_t tw4[4] = {top.x, top.y, top.z, top.w};
        uint32_t sg[8];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const uint32_t tw = tw4[q];
          sg[2 * q] = ((tw << 8) & 0x8000u) | ((tw << 16) & 0x80000000u);
          sg[2 * q + 1] = ((tw >> 8) & 0x8000u) | (tw & 0x80000000u);
        }
        // digit planes of 16 values, most significant first, 4 values per
        // word, with the magnitude shifted right by sh (truncating): whole
        // digits by reading output plane dg from staged plane dg - sh/8 (the
        // top plane without its sign bits; zero above it), then the bit shift
        // within bytes (per-byte masks keep the values of a word apart)
        const int sh = shr[i];
        const int a = sh >> 3, bsh = sh & 7;
        uint32_t m[kDigits][4];
#pragma unroll
        for (int dg = 0; dg < kDigits; ++dg) {
          const int j = dg - a;
          uint4 x4 = make_uint4(0u, 0u, 0u, 0u);
          if (j >= 0) x4 = *reinterpret_cast<const uint4 *>(src + j * KC);
          const uint32_t keep = j == 0 ? 0x7F7F7F7Fu : 0xFFFFFFFFu;
          m[dg][0] = x4.x & keep;
          m[dg][1] = x4.y & keep;
          m[dg][2] = x4.z & keep;
          m[dg][3] = x4.w & keep;
        }
        if (bsh != 0) {
          const uint32_t lo = 0x01010101u * (0xFFu >> bsh);
#pragma unroll
          for (int dg = kDigits - 1; dg >= 1; --dg)
#pragma unroll
            for (int q = 0; q < 4; ++q)
              m[dg][q] = ((m[dg][q] >> bsh) & lo) | ((m[dg - 1][q] << (8 - bsh)) & ~lo);
#pragma unroll
          for (int q = 0; q < 4; ++q) m[0][q] = (m[0][q] >> bsh) & lo;
        }
        const int row = kRowsPerProducer * warp + rl;
        // plane 3: R = X4 + X5 / 256 rounded to FP16: X4 and X5 are exact in
        // FP16 and X5 / 256 too, so one packed FMA rounds the exact sum once
        {
          const __half2 k2m8 = __floats2half2_rn(1.0f / 256.0f, 1.0f / 256.0f);
          uint32_t o[8];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            uint32_t a_lo = __byte_perm(m[3][q], 0x64646464u, 0x4140u);
            uint32_t a_hi = __byte_perm(m[3][q], 0x64646464u, 0x4342u);
            uint32_t b_lo = __byte_perm(m[4][q], 0x64646464u, 0x4140u);
            uint32_t b_hi = __byte_perm(m[4][q], 0x64646464u, 0x4342u);
            const __half2 x4lo = __hsub2(*reinterpret_cast<__half2 *>(&a_lo), k1024);
            const __half2 x4hi = __hsub2(*reinterpret_cast<__half2 *>(&a_hi), k1024);
            const __half2 x5lo = __hsub2(*reinterpret_cast<__half2 *>(&b_lo), k1024);
            const __half2 x5hi = __hsub2(*reinterpret_cast<__half2 *>(&b_hi), k1024);
            __half2 h01 = __hfma2(x5lo, k2m8, x4lo);
            __half2 h23 = __hfma2(x5hi, k2m8, x4hi);
            o[2 * q] = *reinterpret_cast<uint32_t *>(&h01) | sg[2 * q];
            o[2 * q + 1] = *reinterpret_cast<uint32_t *>(&h23) | sg[2 * q + 1];
          }
          uint8_t *pl = xs + 3 * XBYTES;
          *reinterpret_cast<uint4 *>(pl + tc::kmajor_swizzled_offset(row, h * 16, KC)) =
              make_uint4(o[0], o[1], o[2], o[3]);
          *reinterpret_cast<uint4 *>(pl + tc::kmajor_swizzled_offset(row, h * 16 + 8, KC)) =
              make_uint4(o[4], o[5], o[6], o[7]);
        }
        // planes 0..2: the exact digits X1, X2, X3
#pragma unroll
        for (int dg = 0; dg < 3; ++dg) {
          const uint32_t *w = m[dg];
          // bytes (b0, b1) -> FP16 pair (1024 + b0, 1024 + b1) -> minus 1024:
          // exact, two values per packed subtraction
          uint32_t o[8];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            uint32_t lo = __byte_perm(w[q], 0x64646464u, 0x4140u);
            uint32_t hi = __byte_perm(w[q], 0x64646464u, 0x4342u);
            __half2 hlo = __hsub2(*reinterpret_cast<__half2 *>(&lo), k1024);
            __half2 hhi = __hsub2(*reinterpret_cast<__half2 *>(&hi), k1024);
            o[2 * q] = *reinterpret_cast<uint32_t *>(&hlo) | sg[2 * q];
            o[2 * q + 1] = *reinterpret_cast<uint32_t *>(&hhi) | sg[2 * q + 1];
          }
          uint8_t *pl = xs + dg * XBYTES;
          *reinterpret_cast<uint4 *>(pl + tc::kmajor_swizzled_offset(row, h * 16, KC)) =
              make_uint4(o[0], o[1], o[2], o[3]);
          *reinterpret_cast<uint4 *>(pl + tc::kmajor_swizzled_offset(row, h * 16 + 8, KC)) =
              make_uint4(o[4], o[5], o[6], o[7]);
        }
      }
      tc::fence_proxy_async_smem();   // generic writes -> tensor-core reads
      __syncwarp();
      if (lane == 0 && !(withhold && warp == 0 && ubase + v == 0)) mbar_arrive(&bars.xfull[s]);
      return true;
    };
    int u = 0;
    bool aborted = false;
    for (int kidx = k0; kidx < k1 && !aborted; ++kidx) {
      int key = nkey, xr_lane = nxr;
      const int xe_lane = nxe;
      if (kidx + 1 < k1) {
        nkey = p.sched.key_ids[kidx + 1];
        nxr = nnxr;
        nxe = (nxr >= 0 && nxr < p.n_xrows) ? p.x_exp[nxr] : 0;
      }
      if (kidx + 2 < k1) nnxr = p.sched.key_xrow[(int64_t)(kidx + 2) * 128 + my_row];
      const bool key_ok = key >= 0 && key < p.d.n_tables * p.d.n_cases;
      if (!key_ok) {
        if (warp == 0 && lane == 0) report(p.st, VL1_E_ARG, tile, kidx);
        xr_lane = -1;
      }
      if (xr_lane >= p.n_xrows) {
        report(p.st, VL1_E_ARG, tile, my_row);
        xr_lane = -1;
      }
      // a source row above its target row's reference exponent is not one
      // of that row's list-1 sources
      int sh_lane = my_ref - xe_lane;
      if (lane < kRowsPerProducer && xr_lane >= 0 && sh_lane < 0) {
        report(p.st, VL1_E_ARG, tile, my_row);
        xr_lane = -1;
      }
      sh_lane = min(max(sh_lane, 0), kXFixedBits + 1);   // past the width: zero
      const bool key_empty =
          __ballot_sync(0xffffffffu, lane < kRowsPerProducer && xr_lane >= 0) == 0u;
      for (int kc = 0; kc < p.g.n_kc; ++kc, ++u) {
        {
          const int us = u % kStgDepth;
          sh_s0 = us == 0 ? sh_lane : sh_s0;
          sh_s1 = us == 1 ? sh_lane : sh_s1;
          sh_s2 = us == 2 ? sh_lane : sh_s2;
          empty_bits = (empty_bits & ~(1u << us)) | (key_empty ? 1u << us : 0u);
        }
        // gather unit u: piece pc of the warp's rows -> row pc / PPR, piece pc % PPR
        uint8_t *sb = stg + (u % kStgDepth) * kRowsPerProducer * RB;
#pragma unroll
        for (int it = 0; it < (kRowsPerProducer * PPR + 31) / 32; ++it) {
          if (key_empty) break;
          const int pc = it * 32 + lane;
          const int rl = min(pc / PPR, kRowsPerProducer - 1), q = pc - (pc / PPR) * PPR;
          const int xr = __shfl_sync(0xffffffffu, xr_lane, rl);
          if (pc < kRowsPerProducer * PPR) {
            const bool have = xr >= 0;
            const uint8_t *src =
                p.xdig + (have ? (int64_t)xr * row_bytes + (int64_t)kc * RB + q * 16 : 0);
            tc::cp_async16_zfill(sb + rl * RB + q * 16, src, have ? 16u : 0u);
          }
        }
        tc::cp_async_commit();
        if (u >= LOOK) {
          tc::cp_async_wait_group<LOOK>();   // unit u - LOOK landed (this lane's pieces)
          __syncwarp();
          if (!expand(u - LOOK)) {
            aborted = true;
            break;
          }
        }
      }
    }
    tc::cp_async_wait_all();
    __syncwarp();
    for (int v = u - LOOK < 0 ? 0 : u - LOOK; v < u && !aborted; ++v) aborted = !expand(v);
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
        for (int iu = 0; iu < upr; ++iu, ++u) {
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
      tc::tmem_ld16(col, r2);                // i + j = 2: |x| <= 127 * 128 * 64 < 2^20
      tc::tmem_ld16(col + NCH, r3);          // i + j = 3: |x| < 3.2e6 < 2^22
      tc::tmem_ld_wait();
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        // 1.5 * 2^23 + x for |x| < 2^22 is exact, with the integer x in its
        // low bits (raw bits kMagicBits + x); weights 2^16 and 2^8 of the
        // d = 2 and d = 3 terms
        const uint32_t b2 = __float_as_uint(__uint_as_float(r2[c]) + kMagic);
        const uint32_t b3 = __float_as_uint(__uint_as_float(r3[c]) + kMagic);
        acc[c] += (unsigned long long)b2 * 65536ull + (unsigned long long)b3 * 256ull;
      }
      tc::tmem_ld16(col + 2 * NCH, r2);      // i + j = 4: |x| < 5.3e6 < 2^24
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
          acc[c] += (unsigned long long)f32_scaled_to_i64(__uint_as_float(r16[c]), 8);
        tc::tmem_ld16(col + NCH, r16);           // d6, weight 2^32
        tc::tmem_ld_wait();
#pragma unroll
        for (int c = 0; c < 16; ++c)
          acc[c] += (unsigned long long)f32_scaled_to_i64(__uint_as_float(r16[c]), 0);
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
  __shared__ long long s_obase[128];   // result index of the row's first target point
  __shared__ int s_ocnt[128];          // target points of the row's box (0: empty row)
  __shared__ int s_oexp[128];          // an output is (parked sum) * 2^s_oexp
  if (tid < 128) {
    const int v = s_rows[tid];
    int cnt = 0, ex = 0;
    long long ob = 0;
    if (v >= 0) {
      const int j = v / p.nrhs, r = v - (v / p.nrhs) * p.nrhs;
      const int tbox = p.target_boxes[j];
      cnt = min(p.tgt_counts[tbox], p.d.nq);
      ob = (long long)r * p.n_particles + p.tgt_starts[tbox];
      // table values are m_a 2^(a_exp - kFixedBits), densities
      // m_x 2^(e - kXFixedBits) with e the row's reference exponent; the
      // parked sums count units of 2^32 of m_a m_x
      ex = p.a_exp + p.ref_exp[v] - (kFixedBits + kXFixedBits) + 32;
    }
    s_obase[tid] = ob;
    s_ocnt[tid] = cnt;
    s_oexp[tid] = ex;
  }
  const long long *tot_src = reinterpret_cast<const long long *>(smem);
  bool write = !s_abort;
  const uint8_t *g_parts = nullptr;   // slot region of part 0 of a split tile
  const int64_t slot_bytes = (int64_t)128 * NCH * 8;
  const int64_t part_stride = (int64_t)n_chunks * slot_bytes;
  if (item.split >= 0) {
    uint8_t *base = static_cast<uint8_t *>(p.sched.split_partials) +
                    ((int64_t)(item.slot - item.part) * n_chunks + chunk) * slot_bytes;
    g_parts = base;
    if (!s_abort) {
      long long *mine = reinterpret_cast<long long *>(base + item.part * part_stride);
      for (int i = tid; i < 128 * NCH; i += blockDim.x)
        mine[i] = tot_src[(i / NCH) * PARK_STRIDE + i % NCH];
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) {
      // parts count in the low 16 bits; a part that aborted (and stored no
      // partial sums) also adds to the high bits, so that the last part
      // writes nothing for the tile
      const int inc = s_abort ? kSplitPoison + 1 : 1;
      const int done =
          atomicAdd(p.sched.split_counters + item.split * n_chunks + chunk, inc) + inc;
      s_last = (done & (kSplitPoison - 1)) == item.nparts;
      s_poison = done >= kSplitPoison;
    }
    __syncthreads();
    write = write && s_last && !s_poison;
    if (write) __threadfence();
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
          for (int q = 0; q < item.nparts; ++q)
            tot[bi] += __ldcg(reinterpret_cast<const long long *>(g_parts + q * part_stride) + it);
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
  // the last part leaves the counter at zero for the next call (also after
  // an abort, so that a timed-out call does not spoil the schedule)
  if (item.split >= 0 && tid == 0 && s_last)
    p.sched.split_counters[item.split * n_chunks + chunk] = 0;
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
        int *ctr = pj->sched.split_counters + bj.item.split * (pj->g.np / NCH) + bj.chunk;
        const int done = atomicAdd(ctr, kSplitPoison + 1) + kSplitPoison + 1;
        if ((done & (kSplitPoison - 1)) == bj.item.nparts) *ctr = 0;
      }
    }
  }
  ubase += n_rounds * upr;
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
  const size_t pipe = (size_t)kStages * (kXPlanes * 128 + kDigits * nch) * kc * 2 +
                      (size_t)kProducerWarps * kStgDepth * kRowsPerProducer * kDigits * kc;
  const size_t park = (size_t)128 * (nch + 1) * 8;   // int64 sums, padded rows
  return (pipe > park ? pipe : park) + 1024;
}

int mixed_threads(int nch) { return 32 * (kReadWarp0 + 4 * (nch / 16)); }

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
  // above one chunk of 32, K is whole exact rounds of 64
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
  b += (nboxes * nrhs * 4 + 255) / 256 * 256;                    // density row exponents
  b += (n_tgt_boxes * nrhs * 4 + 255) / 256 * 256;               // target row exponents
  b += (nboxes * nrhs * g.kp * kDigits + 255) / 256 * 256;  // x digit bytes
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
  const int64_t n_trows = (int64_t)tree.n_tgt_boxes * nrhs;
  int *x_exp = reinterpret_cast<int *>(w);
  w += (n_xrows * 4 + 255) / 256 * 256;
  int *ref_exp = reinterpret_cast<int *>(w);
  w += (n_trows * 4 + 255) / 256 * 256;
  uint8_t *xdig = w;
  w += (n_xrows * g.kp * kDigits + 255) / 256 * 256;
  double *wbox = nullptr, *disp = nullptr;
  if (d.disp_kind == VL1_DISP_LOG2D) {
    wbox = reinterpret_cast<double *>(w);
    w += (nboxes * nrhs * cv * 8 + 255) / 256 * 256;
    disp = reinterpret_cast<double *>(w);
  }
  cudaError_t e;
  const int64_t nbr = n_xrows;
  // row exponents and digits in one pass, then the target rows' references
  x_digits_kernel<<<grid_for(nbr * 32, 256), 256, 8 * g.kp * kDigits, s>>>(
      d, tree, (int)nboxes, coefs, nrhs, x_exp, xdig, g.kp, g.kc, plan->status);
  ref_exponent_kernel<<<grid_for(n_trows, 256), 256, 0, s>>>(tree, nrhs, x_exp, ref_exp);
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
  mp.xdig = xdig;
  mp.n_xrows = (int32_t)n_xrows;
  mp.adig = plan->mixed.adig;
  mp.x_exp = x_exp;
  mp.ref_exp = ref_exp;
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
  void *d_ttasks = nullptr;   // target-row tasks of the reference exponents
  int n_ttasks = 0;
  std::vector<BatchGroup> groups;
  std::vector<SoloLaunch> solos;
  bool has_disp = false;
  int max_row_bytes = 16;   // largest kp * 5 of the problems (digit staging)
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
    if (ctas >= 2ll * n_sm && n_x < INT32_MAX && mixed_kernel_ptr(g.nch, g.kc, false)) {
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
    const int ctas = ctas_opt > 0 ? ctas_opt : n_sm;
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
    // the workspace layout of launch_mixed: [row exponents][target row
    // exponents][x digits][disp]
    int *x_exp = reinterpret_cast<int *>(w);
    w += round256(L.nrows[i] * 4);
    int *ref_exp = reinterpret_cast<int *>(w);
    w += round256((int64_t)L.preps[i].tr.n_tgt_boxes * q.nrhs * 4);
    uint8_t *xdig = w;
    w += round256(L.nrows[i] * g.kp * kDigits);
    double *wbox = nullptr, *disp = nullptr;
    if (q.plan->d.disp_kind == VL1_DISP_LOG2D) {
      wbox = reinterpret_cast<double *>(w);
      w += round256(L.nrows[i] * cv * 8);
      disp = reinterpret_cast<double *>(w);
      b->has_disp = true;
    }
    L.mps[i].xdig = xdig;
    L.mps[i].x_exp = x_exp;
    L.mps[i].ref_exp = ref_exp;
    L.mps[i].disp = disp;
    L.preps[i].x_exp = x_exp;
    L.preps[i].ref_exp = ref_exp;
    L.preps[i].xdig = xdig;
    b->max_row_bytes = std::max(b->max_row_bytes, g.kp * kDigits);
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
  if (b->n_tasks > 0) {
    x_digits_batch_kernel<<<b->n_tasks, 256, 8 * b->max_row_bytes, s>>>(
        static_cast<const PrepProblem *>(b->d_prep), static_cast<const PrepTask *>(b->d_tasks),
        b->max_row_bytes);
    if (b->n_ttasks > 0)
      ref_exponent_batch_kernel<<<b->n_ttasks, 256, 0, s>>>(
          static_cast<const PrepProblem *>(b->d_prep),
          static_cast<const PrepTask *>(b->d_ttasks));
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
  if (b->n_tasks > 0) n += 1 + (b->n_ttasks > 0 ? 1 : 0);
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
