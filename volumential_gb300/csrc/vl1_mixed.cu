// Mixed-precision list-1 evaluation on the tensor cores (tcgen05, BF16 digits,
// exact FP32 partial products, FP64 final sums).
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
// Exactness (an Ozaki-type split).  A (the blocks, per plan) and x' (per call)
// are written in fixed point against a global power-of-two scale and split
// into ND = 5 signed 8-bit digits, each held exactly in BF16.  A product of
// one digit pair over K <= 64 is an integer below 64*255^2 < 2^22, exact in the
// FP32 accumulator.  Digit pairs (i, j) of weight 2^(-8(i+j)) with i + j <= 4
// (the leading 32 bits) get their own TMEM accumulator, re-initialised per key
// chunk and read after every key chunk into int32 registers (one FADD with
// 1.5 * 2^23 turns the exact float into its integer bits); pairs with
// i + j = 5, 6 accumulate across keys in FP32 TMEM (their rounding is below
// 2^-40 of the result).  The integer diagonals and the two FP32 tails are
// combined in FP64 once per output.
#include <cuda_bf16.h>

#include "vl1_internal.cuh"
#include "vl1_mixed.cuh"
#include "vl1_tc.cuh"

namespace vl1 {

namespace {

constexpr uint32_t kWaitLimit = 1u << 22;
constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
constexpr int kMagicBits = 0x4B400000;

// ----------------------------------------------------------------- helpers

// |v| as a fixed-point integer m with v = sign * 2^(e - 40) * m, m < 2^40,
// rounded to nearest; digits are the five base-256 digits of m.
__device__ __forceinline__ void fixed_digits(double v, int e, int (&dig)[kDigits]) {
  const double sc = ldexp(fabs(v), kFixedBits - e);
  long long m = __double2ll_rn(sc);
  if (m >= (1ll << kFixedBits)) m = (1ll << kFixedBits) - 1;  // v at the scale bound
  const int sgn = v < 0 ? -1 : 1;
#pragma unroll
  for (int i = 0; i < kDigits; ++i) {
    const int shift = kFixedBits - kDigitBits * (i + 1);
    dig[i] = sgn * (int)((m >> shift) & 0xFF);
  }
}

// exponent e with |v| < 2^e (0 for v == 0)
__device__ __forceinline__ int scale_exponent(double v) {
  if (v == 0.0) return -1074;
  int e;
  frexp(fabs(v), &e);
  return e;
}

// ------------------------------------------------- plan: A digit operands

__global__ void build_adig_kernel(DevDesc d, MixedGeom g, __nv_bfloat16 *adig, int a_exp) {
  // element (key, kchunk, digit, n, k) of [key][kchunk][digit][NP][KC]
  // (core-matrix K-major order inside each [NP][KC] tile)
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
    const uint32_t off = tc::kmajor_offset(n, k, g.kc);  // bytes
    adig[tile * per_tile + off / 2] = __int2bfloat16_rn(dig[digit]);
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

// max exponent of scaling * coefficient per rhs
__global__ void x_exponent_kernel(DevDesc d, TreeDev tr, int nboxes, const double *coefs,
                                  int nrhs, int *x_exp) {
  const int64_t n = (int64_t)nboxes * nrhs;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(idx / nrhs), r = (int)(idx % nrhs);
    int cnt = tr.src_counts[b];
    if (cnt <= 0) continue;
    cnt = min(cnt, d.nq);
    const double sc = pair_scaling(d, level_extent(tr.root_extent, tr.levels[b]));
    const double *c = coefs + (int64_t)r * tr.n_particles + tr.src_starts[b];
    int e = -1074;
    for (int s = 0; s < cnt; ++s) e = max(e, scale_exponent(sc * c[s]));
    atomicMax(x_exp + r, e);
  }
}

// x digits: row ((b * kDigits + digit) * nrhs + r), KP bf16 per row, source
// points placed at their mode id; plus one zero row at the end.
__global__ void x_digits_kernel(DevDesc d, TreeDev tr, int nboxes, const double *coefs,
                                int nrhs, const int *x_exp, __nv_bfloat16 *xdig, int kp,
                                int64_t zero_row, vl1_status *st) {
  const int64_t n = (int64_t)nboxes * nrhs;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(idx / nrhs), r = (int)(idx % nrhs);
    int cnt = tr.src_counts[b];
    if (cnt <= 0) continue;
    if (cnt > d.nq) {
      report(st, VL1_E_LAYOUT, b, cnt);
      cnt = d.nq;
    }
    __nv_bfloat16 *rows[kDigits];
#pragma unroll
    for (int i = 0; i < kDigits; ++i) {
      rows[i] = xdig + (((int64_t)b * kDigits + i) * nrhs + r) * kp;
      for (int k = 0; k < kp; ++k) rows[i][k] = __int2bfloat16_rn(0);
    }
    const double sc = pair_scaling(d, level_extent(tr.root_extent, tr.levels[b]));
    const double *c = coefs + (int64_t)r * tr.n_particles + tr.src_starts[b];
    const int e = x_exp[r];
    for (int s = 0; s < cnt; ++s) {
      const int m = tr.smode[tr.src_starts[b] + s];
      if (m < 0 || m >= d.nq) {
        report(st, VL1_E_LAYOUT, b, -1 - s);
        continue;
      }
      int dig[kDigits];
      fixed_digits(sc * c[s], e, dig);
#pragma unroll
      for (int i = 0; i < kDigits; ++i) rows[i][m] = __int2bfloat16_rn(dig[i]);
    }
  }
  if (blockIdx.x == 0)
    for (int k = threadIdx.x; k < kp; k += blockDim.x) xdig[zero_row * kp + k] = __int2bfloat16_rn(0);
}

// 2D log displacement: w[b, r] = dispfac(b) * sum_s nmlz[lev(b), s] * coef
// (complex when the normalizers are), then disp[tb, r] = sum over list 1.
__global__ void disp_box_kernel(DevDesc d, TreeDev tr, int nboxes, const double *coefs,
                                int nrhs, double *w) {
  const int64_t n = (int64_t)nboxes * nrhs;
  const int cv = d.table_cplx ? 2 : 1;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x) {
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
}

__global__ void disp_target_kernel(DevDesc d, TreeDev tr, int nrhs, const double *w,
                                   double *disp) {
  const int64_t n = (int64_t)tr.n_tgt_boxes * nrhs;
  const int cv = d.table_cplx ? 2 : 1;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x) {
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
}

// ---------------------------------------------------------- main kernel

struct MixedParams {
  DevDesc d;
  MixedGeom g;
  int nrhs;
  vl1_mixed_schedule sched;
  const __nv_bfloat16 *xdig;
  int64_t zero_row;
  const __nv_bfloat16 *adig;
  const int *x_exp;
  int a_exp;
  const double *disp;  // [n_tgt_boxes * nrhs] (x2 complex) or nullptr
  const int32_t *target_boxes, *tgt_starts, *tgt_counts;
  int n_tgt_boxes;
  int64_t n_particles;
  double *result;
  vl1_status *st;
};

// digit pairs: 6 exact groups (one pair each) then 2 FP32 tail groups
__constant__ int8_t c_exact_i[6] = {1, 1, 2, 1, 2, 3};
__constant__ int8_t c_exact_j[6] = {1, 2, 1, 3, 2, 1};

template <int NCH>
__global__ void __launch_bounds__(NCH >= 64 ? 256 : 128)
mixed_kernel(const __grid_constant__ MixedParams p) {
  constexpr int NGROUPS = 8;
  // groups at NCH-column strides; a 32-column read of the last group must fit
  constexpr uint32_t TCOLS = NCH * (NGROUPS - 1) + (NCH > 32 ? NCH : 32) <= 256 ? 256 : 512;
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t bar_load, bar_mma;
  __shared__ uint32_t tmem_base;
  __shared__ int s_abort;
  __shared__ int s_rows[128];

  const int KC = p.g.kc;
  const uint32_t xbytes = 128u * KC * 2u;    // one digit of the row operand
  const uint32_t abytes = (uint32_t)NCH * KC * 2u;
  uint8_t *xs = smem;
  uint8_t *as = smem + kDigits * xbytes;

  const int tile = blockIdx.x;
  const int chunk = blockIdx.y;
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int row = ((warp & 3) << 5) | (tid & 31);   // TMEM lane of this thread
  const int wg = tid >> 7;                           // column slice

  if (tid < 128) {
    int v = p.sched.tile_rows[(int64_t)tile * 128 + tid];
    if (v >= (int64_t)p.n_tgt_boxes * p.nrhs) {
      report(p.st, VL1_E_ARG, tile, tid);
      v = -1;
    }
    s_rows[tid] = v;
  }
  if (tid == 0) {
    tc::mbar_init(&bar_load, 1);
    tc::mbar_init(&bar_mma, 1);
    tc::fence_mbar_init();
    s_abort = 0;
  }
  if (warp == 0) {
    tc::tmem_alloc(&tmem_base, TCOLS);
    tc::tmem_relinquish();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tbase = tmem_base;
  const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;

  int acc[3][32];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 32; ++c) acc[a][c] = 0;

  const int k0 = p.sched.tile_key_start[tile], k1 = p.sched.tile_key_start[tile + 1];
  const uint32_t idesc = tc::idesc_bf16_f32(128, NCH);
  const uint32_t sbo = (uint32_t)KC * 16u;
  const int nchunk16 = KC / 8;
  uint32_t phase = 0;
  bool first_unit = true;

  for (int kidx = k0; kidx < k1; ++kidx) {
    const int key = p.sched.key_ids[kidx];
    if (key < 0 || key >= p.d.n_tables * p.d.n_cases) {
      if (tid == 0) report(p.st, VL1_E_ARG, tile, kidx);
      continue;
    }
    for (int kc = 0; kc < p.g.n_kc; ++kc) {
      // ---- stage operands: A digits by bulk copy, X digit rows by cp.async
      if (tid == 0) {
        tc::mbar_arrive_expect_tx(&bar_load, kDigits * abytes);
        const int64_t base = (((int64_t)key * p.g.n_kc + kc) * kDigits) * p.g.np * KC +
                             (int64_t)chunk * NCH * KC;
        for (int dg = 0; dg < kDigits; ++dg)
          tc::bulk_g2s(as + dg * abytes, p.adig + base + (int64_t)dg * p.g.np * KC, abytes,
                       &bar_load);
      }
      const int n_items = 128 * kDigits * nchunk16;
      for (int it = tid; it < n_items; it += blockDim.x) {
        const int c16 = it % nchunk16;
        const int rd = it / nchunk16;
        const int r = rd & 127;
        const int dg = rd >> 7;
        const int xr = p.sched.key_xrow[(int64_t)kidx * 128 + r];
        const bool valid = xr >= 0 && (int64_t)xr + (int64_t)(kDigits - 1) * p.nrhs < p.zero_row;
        if (xr >= 0 && !valid && dg == 0 && c16 == 0) report(p.st, VL1_E_ARG, tile, r);
        const int64_t src_row = valid ? (int64_t)xr + (int64_t)dg * p.nrhs : p.zero_row;
        tc::cp_async16(xs + dg * xbytes + tc::kmajor_offset(r, c16 * 8, KC),
                       p.xdig + src_row * p.g.kp + kc * KC + c16 * 8);
      }
      tc::cp_async_commit();
      tc::cp_async_wait_all();
      if (!tc::mbar_wait_bounded(&bar_load, phase, kWaitLimit)) s_abort = 1;
      tc::fence_proxy_async_smem();
      tc::tc_fence_before();
      __syncthreads();
      tc::tc_fence_after();
      if (s_abort) break;

      // ---- tensor-core products
      if (tid == 0) {
        const uint32_t xa = tc::smem_addr(xs), aa = tc::smem_addr(as);
        for (int g = 0; g < NGROUPS; ++g) {
          const uint32_t dcol = tbase + (uint32_t)(g * NCH);
          bool first = true;
          // exact groups: one pair; tails: pairs with i + j = 5 (g = 6), 6 (g = 7)
          const int diag = g < 6 ? 0 : g - 1;
          const int np_ = g < 6 ? 1 : diag - 1;
          for (int q = 0; q < np_; ++q) {
            const int i = g < 6 ? c_exact_i[g] : q + 1;
            const int j = g < 6 ? c_exact_j[g] : diag - q - 1;
            for (int kk = 0; kk < KC / 16; ++kk) {
              const uint64_t ad = tc::smem_desc_kmajor_noswizzle(
                  xa + (uint32_t)(i - 1) * xbytes + kk * 256u, 128u, sbo);
              const uint64_t bd = tc::smem_desc_kmajor_noswizzle(
                  aa + (uint32_t)(j - 1) * abytes + kk * 256u, 128u, sbo);
              const uint32_t accumulate = g < 6 ? !first : !(first && first_unit);
              tc::mma_bf16(dcol, ad, bd, idesc, accumulate);
              first = false;
            }
          }
        }
        tc::mma_commit(&bar_mma);
      }
      if (!tc::mbar_wait_bounded(&bar_mma, phase, kWaitLimit)) s_abort = 1;
      tc::tc_fence_after();
      __syncthreads();
      if (s_abort) break;

      // ---- exact groups: integer accumulation
#pragma unroll
      for (int g = 0; g < 6; ++g) {
        uint32_t r32[32];
        tc::tmem_ld32(tbase + lane_off + (uint32_t)(g * NCH + wg * 32), r32);
        tc::tmem_ld_wait();
        const int a = g == 0 ? 0 : (g <= 2 ? 1 : 2);   // i + j - 2 of the pair
#pragma unroll
        for (int c = 0; c < 32; ++c)
          acc[a][c] += __float_as_int(__uint_as_float(r32[c]) + kMagic) - kMagicBits;
      }
      tc::tc_fence_before();
      __syncthreads();
      tc::tc_fence_after();
      phase ^= 1u;
      first_unit = false;
    }
    if (s_abort) break;
  }

  if (!s_abort) {
    // ---- FP32 tails (weights 2^-40 and 2^-48 of the scale); a tile without
    // keys has only zero (plus displacement) outputs
    float tail[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) tail[c] = 0.0f;
#pragma unroll
    for (int g = 6; g < 8; ++g) {
      if (k1 == k0) break;
      uint32_t r32[32];
      tc::tmem_ld32(tbase + lane_off + (uint32_t)(g * NCH + wg * 32), r32);
      tc::tmem_ld_wait();
      const float wgt = g == 6 ? 1.0f : 1.0f / 256.0f;
#pragma unroll
      for (int c = 0; c < 32; ++c) tail[c] += __uint_as_float(r32[c]) * wgt;
    }
    const int v = s_rows[row];
    if (v >= 0) {
      const int j = v / p.nrhs, r = v % p.nrhs;
      const int tbox = p.target_boxes[j];
      const int tbeg = p.tgt_starts[tbox];
      const int ntgt = min(p.tgt_counts[tbox], p.d.nq);
      const int e = p.a_exp + p.x_exp[r];
      const double w2 = ldexp(1.0, e - 16), w3 = ldexp(1.0, e - 24),
                   w4 = ldexp(1.0, e - 32), w5 = ldexp(1.0, e - 40);
      const bool oc = p.d.table_cplx;
      double disp_re = 0.0, disp_im = 0.0;
      if (p.disp) {
        const int64_t di = (int64_t)j * p.nrhs + r;
        disp_re = oc ? p.disp[2 * di] : p.disp[di];
        disp_im = oc ? p.disp[2 * di + 1] : 0.0;
      }
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        const int n = chunk * NCH + wg * 32 + c;
        if (wg * 32 + c >= NCH) break;
        int t = n, part = 0;
        if (oc && n >= p.d.nq) {
          t = n - p.d.nq;
          part = 1;
        }
        if (t >= ntgt || n >= (oc ? 2 * p.d.nq : p.d.nq)) continue;
        double y = (double)acc[0][c] * w2 + (double)acc[1][c] * w3 +
                   (double)acc[2][c] * w4 + (double)tail[c] * w5;
        y += part ? disp_im : disp_re;
        const int64_t o = (int64_t)r * p.n_particles + tbeg + t;
        if (oc)
          p.result[2 * o + part] = y;
        else
          p.result[o] = y;
      }
    }
  }
  if (s_abort && tid == 0) {
    // give in-flight copies and products a bounded chance to land before the
    // accumulators are released
    tc::mbar_wait_bounded(&bar_load, phase, kWaitLimit);
    tc::mbar_wait_bounded(&bar_mma, phase, kWaitLimit);
    report(p.st, VL1_E_TIMEOUT, tile, chunk);
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, TCOLS);
}

int grid_for(int64_t n, int threads) {
  int64_t g = (n + threads - 1) / threads;
  if (g > 152 * 32) g = 152 * 32;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace

MixedGeom mixed_geometry(int nq, int table_cplx) {
  MixedGeom g;
  g.kp = ((nq + 15) / 16) * 16;
  g.kc = g.kp <= 64 ? g.kp : 64;
  g.kp = ((g.kp + g.kc - 1) / g.kc) * g.kc;
  g.n_kc = g.kp / g.kc;
  const int n = table_cplx ? 2 * nq : nq;
  g.np = ((n + 15) / 16) * 16;
  if (g.np <= 16) {
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
  MixedGeom g = mixed_geometry(d.nq, d.table_cplx);
  int e = 0;
  if (table_absmax > 0) frexp(table_absmax, &e);
  plan->mixed.geom = g;
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
  b += ((int64_t)nrhs * 4 + 255) / 256 * 256;                   // x exponents
  b += ((nboxes * kDigits * nrhs + 1) * g.kp * 2 + 255) / 256 * 256;  // x digits
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
  uint8_t *w = static_cast<uint8_t *>(workspace);
  int *x_exp = reinterpret_cast<int *>(w);
  const int64_t exp_bytes = ((int64_t)nrhs * 4 + 255) / 256 * 256;
  w += exp_bytes;
  __nv_bfloat16 *xdig = reinterpret_cast<__nv_bfloat16 *>(w);
  const int64_t zero_row = nboxes * kDigits * nrhs;
  w += ((zero_row + 1) * g.kp * 2 + 255) / 256 * 256;
  double *wbox = nullptr, *disp = nullptr;
  if (d.disp_kind == VL1_DISP_LOG2D) {
    wbox = reinterpret_cast<double *>(w);
    w += (nboxes * nrhs * cv * 8 + 255) / 256 * 256;
    disp = reinterpret_cast<double *>(w);
  }
  cudaError_t e = cudaMemsetAsync(x_exp, 0x80, exp_bytes, s);  // large negative exponents
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(x_exp)");
  const int64_t nbr = nboxes * nrhs;
  x_exponent_kernel<<<grid_for(nbr, 256), 256, 0, s>>>(d, tree, (int)nboxes, coefs, nrhs,
                                                      x_exp);
  x_digits_kernel<<<grid_for(nbr, 128), 128, 0, s>>>(d, tree, (int)nboxes, coefs, nrhs, x_exp,
                                                    xdig, g.kp, zero_row, plan->status);
  if (disp) {
    disp_box_kernel<<<grid_for(nbr, 256), 256, 0, s>>>(d, tree, (int)nboxes, coefs, nrhs,
                                                      wbox);
    disp_target_kernel<<<grid_for((int64_t)tree.n_tgt_boxes * nrhs, 256), 256, 0, s>>>(
        d, tree, nrhs, wbox, disp);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "mixed preparation launch");
  if (sched.n_tiles == 0) return VL1_OK;

  MixedParams mp;
  mp.d = d;
  mp.g = g;
  mp.nrhs = nrhs;
  mp.sched = sched;
  mp.xdig = xdig;
  mp.zero_row = zero_row;
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
  const size_t smem = (size_t)kDigits * (128 + g.nch) * g.kc * 2;
  dim3 grid(sched.n_tiles, g.np / g.nch);
  if (g.nch == 64) {
    cudaFuncSetAttribute(mixed_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    mixed_kernel<64><<<grid, 256, smem, s>>>(mp);
  } else if (g.nch == 32) {
    cudaFuncSetAttribute(mixed_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    mixed_kernel<32><<<grid, 128, smem, s>>>(mp);
  } else {
    cudaFuncSetAttribute(mixed_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    mixed_kernel<16><<<grid, 128, smem, s>>>(mp);
  }
  e = cudaGetLastError();
  return e == cudaSuccess ? VL1_OK : cuda_fail(e, "mixed_kernel launch");
}

}  // namespace vl1
