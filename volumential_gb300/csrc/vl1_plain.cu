// Plain FP64 list-1 evaluation and the per-plan block expansion.
//
// The reference's near_field kernel (volumential/list1.py:1050-1159) walks,
// for every target point, every list-1 source box and every source point, and
// recomputes the case id, the table level, the scaling, the log displacement
// and the integer orbit row of the pair.  Here:
//
//  * the integer orbit row and sign of every (table level, case, source mode,
//    target point) are computed once per plan by expand_blocks_kernel into a
//    dense block per (level, case), [source mode][target point], sign applied;
//  * one CTA per (target box, right-hand side) computes the case id, table
//    level, scaling and displacement factor of each of its list-1 pairs once
//    (bit-exact case encoding, vl1_internal.cuh), stages the pair's source
//    coefficients (pre-multiplied by the scaling) in shared memory, and
//    every thread accumulates one target point over a strided subset of the
//    source points with FP64 FMAs, reading block rows with coalesced loads
//    (consecutive threads = consecutive target points);
//  * the 2D log displacement, which does not depend on the target point,
//    is reduced once per target box (warp shuffles) and added to all its
//    targets;
//  * partial sums of the source split are combined through shared memory.
#include <cmath>

#include "vl1_internal.cuh"

namespace vl1 {

namespace {

struct PairInfo {
  int blk;       // element offset of the (level, case) block
  int src_beg;   // first particle of the source box
  int nsrc;      // valid source points (0 if the pair is invalid)
  int lev;       // table level
  double scaling;
  double dispfac;  // disp_coef * scaling * log(ext / table_root_extent)
};

constexpr int kMaxPairChunk = 64;

__global__ void expand_blocks_kernel(DevDesc d, double *blocks, int64_t n_elems,
                                     vl1_status *st) {
  const int nq = d.nq;
  const int64_t per_level = (int64_t)d.n_cases * nq * nq;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n_elems;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int t = (int)(idx % nq);
    const int s = (int)((idx / nq) % nq);
    const int64_t lc = idx / ((int64_t)nq * nq);
    const int c = (int)(lc % d.n_cases);
    const int lev = (int)(idx / per_level);
    int row, sign;
    orbit_row(d, c, s, t, row, sign);
    double re = 0.0, im = 0.0;
    if (row < 0 || row >= d.n_entries) {
      report(st, VL1_E_ENTRY_OOB, c, row);
    } else if (d.table_cplx) {
      re = d.table[2 * ((int64_t)lev * d.n_entries + row)] * (double)sign;
      im = d.table[2 * ((int64_t)lev * d.n_entries + row) + 1] * (double)sign;
    } else {
      re = d.table[(int64_t)lev * d.n_entries + row] * (double)sign;
    }
    if (d.table_cplx) {
      blocks[2 * idx] = re;
      blocks[2 * idx + 1] = im;
    } else {
      blocks[idx] = re;
    }
  }
}

__global__ void index_map_kernel(DevDesc d, int32_t *rows, int8_t *signs) {
  const int nq = d.nq;
  const int64_t n = (int64_t)d.n_cases * nq * nq;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int t = (int)(idx % nq);
    const int s = (int)((idx / nq) % nq);
    const int c = (int)(idx / ((int64_t)nq * nq));
    int row, sign;
    orbit_row(d, c, s, t, row, sign);
    rows[idx] = row;
    signs[idx] = (int8_t)sign;
  }
}

template <bool TC, bool CC>
__global__ void __launch_bounds__(256)
plain_kernel(DevDesc d, TreeDev tr, const double *__restrict__ coefs,
             double *__restrict__ result, int split, int pch, vl1_status *st) {
  constexpr bool OC = TC || CC;
  constexpr int CV = CC ? 2 : 1;  // doubles per coefficient
  constexpr int OV = OC ? 2 : 1;  // doubles per output
  constexpr int TV = TC ? 2 : 1;  // doubles per block value

  extern __shared__ __align__(16) unsigned char smem[];
  const int nq = d.nq;
  PairInfo *info = reinterpret_cast<PairInfo *>(smem);
  double *cs = reinterpret_cast<double *>(info + pch);          // [pch][nq][CV]
  double *red = cs + (size_t)pch * nq * CV;                      // [split][nq][OV]
  double *dsum = red + (size_t)split * nq * OV;                  // [32][OV]
  short *sm = reinterpret_cast<short *>(dsum + 32 * OV);         // [pch][nq]

  const int tb = blockIdx.x;
  const int rhs = blockIdx.y;
  const int64_t rhs_off = (int64_t)rhs * tr.n_particles;
  const int tbox_id = tr.target_boxes[tb];
  const int tbeg = tr.tgt_starts[tbox_id];
  int ntgt = tr.tgt_counts[tbox_id];
  if (ntgt > nq) {
    if (threadIdx.x == 0) report(st, VL1_E_LAYOUT, tb, ntgt);
    ntgt = nq;
  }
  const int p_begin = tr.starts[tb], p_end = tr.starts[tb + 1];

  const int item = threadIdx.x;
  const int t = item % nq;
  const int sg = item / nq;
  const bool active = sg < split;
  int tm = -1;
  if (active && t < ntgt) {
    tm = tr.tmode[tbeg + t];
    if (tm < 0 || tm >= nq) {
      report(st, VL1_E_LAYOUT, tb, -1 - t);
      tm = -1;
    }
  }

  double acc_re = 0.0, acc_im = 0.0;
  double dre = 0.0, dim_ = 0.0;

  for (int p0 = p_begin; p0 < p_end; p0 += pch) {
    const int np = min(pch, p_end - p0);
    // -- per-pair quantities, once per (target box, source box)
    for (int i = threadIdx.x; i < np; i += blockDim.x) {
      const int sbox = tr.lists[p0 + i];
      const int lvl = tr.levels[sbox];
      const double ext = level_extent(tr.root_extent, lvl);
      const int c = pair_case_id(d, tr, tbox_id, sbox, ext);
      PairInfo pi;
      pi.lev = pair_table_level(d, lvl);
      pi.scaling = pair_scaling(d, ext);
      pi.dispfac = 0.0;
      if (d.disp_kind == VL1_DISP_LOG2D)
        pi.dispfac = __dmul_rn(__dmul_rn(d.disp_coef, pi.scaling),
                               log(__ddiv_rn(ext, d.table_root_extent)));
      pi.src_beg = tr.src_starts[sbox];
      pi.nsrc = tr.src_counts[sbox];
      if (pi.nsrc > nq) {
        report(st, VL1_E_LAYOUT, tb, p0 + i);
        pi.nsrc = nq;
      }
      if (c < 0) {
        report(st, VL1_E_INVALID_CASE, tb, p0 + i);
        pi.nsrc = 0;
        pi.blk = 0;
      } else {
        pi.blk = (int)(((int64_t)pi.lev * d.n_cases + c) * nq * nq);
      }
      info[i] = pi;
    }
    __syncthreads();

    // -- stage scaled coefficients and source modes; displacement partials
    for (int k = threadIdx.x; k < np * nq; k += blockDim.x) {
      const int i = k / nq;
      const int sid = k - i * nq;
      const PairInfo &pi = info[i];
      double c_re = 0.0, c_im = 0.0;
      short mode = 0;
      if (sid < pi.nsrc) {
        const int src = pi.src_beg + sid;
        const int m = tr.smode[src];
        if (m < 0 || m >= nq) {
          report(st, VL1_E_LAYOUT, tb, p0 + i);
        } else {
          mode = (short)m;
          if (CC) {
            c_re = coefs[2 * (rhs_off + src)];
            c_im = coefs[2 * (rhs_off + src) + 1];
          } else {
            c_re = coefs[rhs_off + src];
          }
          if (d.disp_kind == VL1_DISP_LOG2D) {
            const int64_t ni = (int64_t)pi.lev * nq + sid;
            const double n_re = TC ? d.nmlz[2 * ni] : d.nmlz[ni];
            const double n_im = TC ? d.nmlz[2 * ni + 1] : 0.0;
            const double w_re = pi.dispfac * n_re, w_im = pi.dispfac * n_im;
            dre += c_re * w_re - c_im * w_im;
            dim_ += c_re * w_im + c_im * w_re;
          }
        }
      }
      cs[(size_t)k * CV] = c_re * pi.scaling;
      if (CC) cs[(size_t)k * CV + 1] = c_im * pi.scaling;
      sm[k] = mode;
    }
    __syncthreads();

    // -- FP64 block products
    if (active && tm >= 0) {
      for (int i = 0; i < np; ++i) {
        const PairInfo &pi = info[i];
        const double *__restrict__ B = d.blocks + (size_t)TV * ((size_t)pi.blk + tm);
        const double *csi = cs + (size_t)i * nq * CV;
        const short *smi = sm + i * nq;
        for (int sid = sg; sid < pi.nsrc; sid += split) {
          const size_t off = (size_t)TV * ((size_t)smi[sid] * nq);
          if (TC && CC) {
            const double b_re = __ldg(B + off), b_im = __ldg(B + off + 1);
            const double a_re = csi[2 * sid], a_im = csi[2 * sid + 1];
            acc_re = fma(a_re, b_re, acc_re);
            acc_re = fma(-a_im, b_im, acc_re);
            acc_im = fma(a_re, b_im, acc_im);
            acc_im = fma(a_im, b_re, acc_im);
          } else if (TC) {
            const double a = csi[sid];
            acc_re = fma(a, __ldg(B + off), acc_re);
            acc_im = fma(a, __ldg(B + off + 1), acc_im);
          } else if (CC) {
            const double b = __ldg(B + off);
            acc_re = fma(csi[2 * sid], b, acc_re);
            acc_im = fma(csi[2 * sid + 1], b, acc_im);
          } else {
            acc_re = fma(csi[sid], __ldg(B + off), acc_re);
          }
        }
      }
    }
    __syncthreads();
  }

  // -- displacement: block-wide sum (warp shuffles, then one warp)
  if (d.disp_kind == VL1_DISP_LOG2D) {
    for (int o = 16; o > 0; o >>= 1) {
      dre += __shfl_xor_sync(0xffffffffu, dre, o);
      if (OC) dim_ += __shfl_xor_sync(0xffffffffu, dim_, o);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
      dsum[warp * OV] = dre;
      if (OC) dsum[warp * OV + 1] = dim_;
    }
    __syncthreads();
    if (warp == 0) {
      const int nw = (blockDim.x + 31) >> 5;
      dre = lane < nw ? dsum[lane * OV] : 0.0;
      dim_ = (OC && lane < nw) ? dsum[lane * OV + 1] : 0.0;
      for (int o = 16; o > 0; o >>= 1) {
        dre += __shfl_xor_sync(0xffffffffu, dre, o);
        if (OC) dim_ += __shfl_xor_sync(0xffffffffu, dim_, o);
      }
      if (lane == 0) {
        dsum[0] = dre;
        if (OC) dsum[1] = dim_;
      }
    }
    __syncthreads();
    dre = dsum[0];
    dim_ = OC ? dsum[1] : 0.0;
  }

  // -- combine the source split and write
  if (active) {
    red[(size_t)(sg * nq + t) * OV] = acc_re;
    if (OC) red[(size_t)(sg * nq + t) * OV + 1] = acc_im;
  }
  __syncthreads();
  if (active && sg == 0 && t < ntgt) {
    double r_re = 0.0, r_im = 0.0;
    for (int g = 0; g < split; ++g) {
      r_re += red[(size_t)(g * nq + t) * OV];
      if (OC) r_im += red[(size_t)(g * nq + t) * OV + 1];
    }
    if (tm < 0) {
      r_re = 0.0;
      r_im = 0.0;
    } else {
      r_re += dre;
      r_im += dim_;
    }
    const int64_t o = rhs_off + tbeg + t;
    if (OC) {
      result[2 * o] = r_re;
      result[2 * o + 1] = r_im;
    } else {
      result[o] = r_re;
    }
  }
}

int grid_for(int64_t n, int threads) {
  int64_t g = (n + threads - 1) / threads;
  if (g > 152 * 64) g = 152 * 64;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace

int32_t launch_expand_blocks(vl1_plan *plan, cudaStream_t s) {
  const int threads = 256;
  expand_blocks_kernel<<<grid_for(plan->block_elems, threads), threads, 0, s>>>(
      plan->d, const_cast<double *>(plan->d.blocks), plan->block_elems, plan->status);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? VL1_OK : cuda_fail(e, "expand_blocks_kernel launch");
}

int32_t launch_index_map(vl1_plan *plan, int32_t *rows, int8_t *signs, cudaStream_t s) {
  const int64_t n = (int64_t)plan->d.n_cases * plan->d.nq * plan->d.nq;
  const int threads = 256;
  index_map_kernel<<<grid_for(n, threads), threads, 0, s>>>(plan->d, rows, signs);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? VL1_OK : cuda_fail(e, "index_map_kernel launch");
}

int32_t launch_plain(vl1_plan *plan, const TreeDev &tree, const double *coefs,
                     int coef_cplx, int nrhs, double *result, cudaStream_t s) {
  const DevDesc &d = plan->d;
  const int nq = d.nq;
  int split = (int)lround(128.0 / nq);
  split = split < 1 ? 1 : (split > 8 ? 8 : split);
  if (split > nq) split = nq;
  int threads = ((nq * split + 31) / 32) * 32;
  if (threads > 256) {
    set_error("q^dim = %d too large for the plain kernel", nq);
    return VL1_E_UNSUPPORTED;
  }
  const int tc = d.table_cplx, cc = coef_cplx;
  const int ov = (tc || cc) ? 2 : 1, cv = cc ? 2 : 1;
  int pch = (int)(32768 / ((size_t)nq * (8 * cv + 2)));
  pch = pch < 1 ? 1 : (pch > kMaxPairChunk ? kMaxPairChunk : pch);
  const size_t smem = sizeof(PairInfo) * pch + sizeof(double) * (size_t)pch * nq * cv +
                      sizeof(double) * (size_t)split * nq * ov + sizeof(double) * 32 * ov +
                      sizeof(short) * (size_t)pch * nq;
  if (smem > 48 * 1024) {
    set_error("plain kernel shared memory %zu exceeds 48 KiB", smem);
    return VL1_E_UNSUPPORTED;
  }
  dim3 grid(tree.n_tgt_boxes, nrhs);
  if (nrhs > 65535) {
    set_error("nrhs %d exceeds 65535", nrhs);
    return VL1_E_ARG;
  }
  if (tc && cc)
    plain_kernel<true, true><<<grid, threads, smem, s>>>(d, tree, coefs, result, split, pch, plan->status);
  else if (tc)
    plain_kernel<true, false><<<grid, threads, smem, s>>>(d, tree, coefs, result, split, pch, plan->status);
  else if (cc)
    plain_kernel<false, true><<<grid, threads, smem, s>>>(d, tree, coefs, result, split, pch, plan->status);
  else
    plain_kernel<false, false><<<grid, threads, smem, s>>>(d, tree, coefs, result, split, pch, plan->status);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? VL1_OK : cuda_fail(e, "plain_kernel launch");
}

}  // namespace vl1
