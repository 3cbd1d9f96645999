// Helmholtz split correction: the list-1 point-to-point sum of the smooth
// remainder R = G_k - G_0 (Helmholtz minus Laplace), which the split mode
// adds to the Laplace-table near field
// (volumential/expansion_wrangler_fpnd.py:3491-3836, split order 1: the
// series remainder kernel of :212-332, strengths = density x quadrature
// weight, self pairs excluded by default).
//
//   2D: R(r) = c0 + sum_{n=1..N} (a_n log r + b_n) r^{2n}
//   3D: R(r) = sum_{n=1..N} c_n r^{n-1}
//
// with complex coefficients computed on the host.  One CTA per target box,
// one thread per target point; the points and strengths of each list-1
// source box are staged in shared memory.  FP64 throughout (the remainder
// sum is FP64-pipe bound: ~2N complex FMAs plus a log per pair in 2D).

#include <cuda_runtime.h>

#include <cstdint>

#include "vl1_internal.cuh"

namespace vl1 {
namespace {

constexpr int kSplitThreads = 128;
constexpr int kSplitMaxTerms = 128;

struct SplitArgs {
  int dim, n_points, nmax, exclude_self, wcplx, n_tgt_boxes;
  // 1: real wave number.  2D: the a_n are real and Im b_n = rho a_n, so two
  // real Horner sums give R; 3D: c_n is real for even n and imaginary for
  // odd n, so Re R and Im R are two Horner sums in r^2 over half the terms
  int real_k;
  double rho;
  const int32_t *target_boxes, *starts, *lists;
  const int32_t *src_starts, *src_counts, *tgt_starts, *tgt_counts;
  const double *points;    // [dim][n_points]
  const double *weights;   // [n_points] or [n_points][2]
  const double *coef;      // [2][nmax + 1][2]: (a_n | c_n) then (b_n), (re, im); index 0: c0
  double *result;          // [n_points][2]
};

template <int DIM>
__global__ void __launch_bounds__(kSplitThreads) split_remainder_kernel(const SplitArgs A) {
  __shared__ double s_pts[DIM][kSplitThreads];
  __shared__ double s_w[2][kSplitThreads];
  __shared__ int s_idx[kSplitThreads];
  __shared__ double s_coef[2][kSplitMaxTerms + 1][2];
  for (int i = threadIdx.x; i < 2 * (A.nmax + 1); i += blockDim.x) {
    const int part = i / (A.nmax + 1), n = i - part * (A.nmax + 1);
    s_coef[part][n][0] = A.coef[(part * (A.nmax + 1) + n) * 2];
    s_coef[part][n][1] = A.coef[(part * (A.nmax + 1) + n) * 2 + 1];
  }
  __syncthreads();
  const int tb = A.target_boxes[blockIdx.x];
  const int t0 = A.tgt_starts[tb], nt = A.tgt_counts[tb];
  for (int tbase = 0; tbase < nt; tbase += kSplitThreads) {
    const int ti = tbase + threadIdx.x;
    const bool have_t = ti < nt;
    const int tgt = have_t ? t0 + ti : 0;
    double x[DIM];
#pragma unroll
    for (int a = 0; a < DIM; ++a) x[a] = have_t ? A.points[(int64_t)a * A.n_points + tgt] : 0.0;
    double acc_re = 0.0, acc_im = 0.0;
    for (int p = A.starts[blockIdx.x]; p < A.starts[blockIdx.x + 1]; ++p) {
      const int sb = A.lists[p];
      const int s0 = A.src_starts[sb], ns = A.src_counts[sb];
      for (int sbase = 0; sbase < ns; sbase += kSplitThreads) {
        const int m = min(kSplitThreads, ns - sbase);
        __syncthreads();
        if (threadIdx.x < m) {
          const int s = s0 + sbase + threadIdx.x;
#pragma unroll
          for (int a = 0; a < DIM; ++a) s_pts[a][threadIdx.x] = A.points[(int64_t)a * A.n_points + s];
          s_w[0][threadIdx.x] = A.wcplx ? A.weights[2 * (int64_t)s] : A.weights[s];
          s_w[1][threadIdx.x] = A.wcplx ? A.weights[2 * (int64_t)s + 1] : 0.0;
          s_idx[threadIdx.x] = s;
        }
        __syncthreads();
        if (!have_t) continue;
        for (int j = 0; j < m; ++j) {
          if (A.exclude_self && s_idx[j] == tgt) continue;
          double r2 = 0.0;
#pragma unroll
          for (int a = 0; a < DIM; ++a) {
            const double d = x[a] - s_pts[a][j];
            r2 = fma(d, d, r2);
          }
          double re, im;
          if (DIM == 2 && A.real_k) {
            double pa = s_coef[0][A.nmax][0], pb = s_coef[1][A.nmax][0];
            for (int n = A.nmax - 1; n >= 1; --n) {
              pa = fma(pa, r2, s_coef[0][n][0]);
              pb = fma(pb, r2, s_coef[1][n][0]);
            }
            const double lg = r2 > 0.0 ? 0.5 * log(r2) : 0.0;
            re = s_coef[0][0][0] + r2 * fma(lg, pa, pb);
            im = fma(A.rho * r2, pa, s_coef[0][0][1]);
          } else if (DIM == 3 && A.real_k) {
            const double r = sqrt(r2);
            // Re R = r sum_{m>=1} c_{2m} r2^(m-1), Im R = sum_{m>=0} Im c_{2m+1} r2^m
            const int me = A.nmax / 2, mo = (A.nmax - 1) / 2;
            double pe = me >= 1 ? s_coef[0][2 * me][0] : 0.0;
            for (int m = me - 1; m >= 1; --m) pe = fma(pe, r2, s_coef[0][2 * m][0]);
            double po = s_coef[0][2 * mo + 1][1];
            for (int m = mo - 1; m >= 0; --m) po = fma(po, r2, s_coef[0][2 * m + 1][1]);
            re = r * pe;
            im = po;
          } else if (DIM == 2) {
            // Horner in x = r^2 for the log and power series (terms n >= 1)
            double pa_re = s_coef[0][A.nmax][0], pa_im = s_coef[0][A.nmax][1];
            double pb_re = s_coef[1][A.nmax][0], pb_im = s_coef[1][A.nmax][1];
            for (int n = A.nmax - 1; n >= 1; --n) {
              pa_re = fma(pa_re, r2, s_coef[0][n][0]);
              pa_im = fma(pa_im, r2, s_coef[0][n][1]);
              pb_re = fma(pb_re, r2, s_coef[1][n][0]);
              pb_im = fma(pb_im, r2, s_coef[1][n][1]);
            }
            // the log term is dropped at r = 0 (its factor r^{2n} vanishes;
            // any nonzero r2 in FP64 has r far above 1e-300)
            const double lg = r2 > 0.0 ? 0.5 * log(r2) : 0.0;
            re = s_coef[0][0][0] + r2 * fma(lg, pa_re, pb_re);
            im = s_coef[0][0][1] + r2 * fma(lg, pa_im, pb_im);
          } else {
            const double r = sqrt(r2);
            re = s_coef[0][A.nmax][0];
            im = s_coef[0][A.nmax][1];
            for (int n = A.nmax - 1; n >= 1; --n) {
              re = fma(re, r, s_coef[0][n][0]);
              im = fma(im, r, s_coef[0][n][1]);
            }
          }
          const double wr = s_w[0][j], wi = s_w[1][j];
          acc_re = fma(wr, re, fma(-wi, im, acc_re));
          acc_im = fma(wr, im, fma(wi, re, acc_im));
        }
      }
    }
    if (have_t) {
      A.result[2 * (int64_t)tgt] = acc_re;
      A.result[2 * (int64_t)tgt + 1] = acc_im;
    }
  }
}

}  // namespace
}  // namespace vl1

using namespace vl1;

extern "C" int32_t vl1_split_correction(const vl1_split_desc *desc, void *stream) {
  if (!desc || !desc->tree || !desc->points || !desc->weights || !desc->coefficients ||
      !desc->result) {
    set_error("vl1_split_correction: null argument");
    return VL1_E_ARG;
  }
  const vl1_split_desc &D = *desc;
  const vl1_tree_view &T = *D.tree;
  if ((D.dim != 2 && D.dim != 3) || D.n_points < 0 || D.n_terms < 1 ||
      D.n_terms > kSplitMaxTerms || T.n_target_boxes < 0) {
    set_error("vl1_split_correction: dim %d, %d points or %d series terms out of range",
              D.dim, D.n_points, D.n_terms);
    return VL1_E_ARG;
  }
  if (T.n_target_boxes == 0) return VL1_OK;
  if (!T.target_boxes || !T.neighbor_source_boxes_starts || !T.neighbor_source_boxes_lists ||
      !T.box_source_starts || !T.box_source_counts_nonchild || !T.box_target_starts ||
      !T.box_target_counts_nonchild) {
    set_error("vl1_split_correction: null array in the tree view");
    return VL1_E_ARG;
  }
  SplitArgs A;
  A.dim = D.dim;
  A.n_points = D.n_points;
  A.nmax = D.n_terms;
  A.exclude_self = D.exclude_self;
  A.wcplx = D.weights_complex;
  A.n_tgt_boxes = T.n_target_boxes;
  A.real_k = (D.flags & VL1_SPLIT_REAL_K) ? 1 : 0;
  A.rho = -0.5 * 3.14159265358979323846;   // Im b_n / a_n for a real wave number
  A.target_boxes = T.target_boxes;
  A.starts = T.neighbor_source_boxes_starts;
  A.lists = T.neighbor_source_boxes_lists;
  A.src_starts = T.box_source_starts;
  A.src_counts = T.box_source_counts_nonchild;
  A.tgt_starts = T.box_target_starts;
  A.tgt_counts = T.box_target_counts_nonchild;
  A.points = D.points;
  A.weights = D.weights;
  A.coef = D.coefficients;
  A.result = D.result;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (D.dim == 2)
    split_remainder_kernel<2><<<T.n_target_boxes, kSplitThreads, 0, s>>>(A);
  else
    split_remainder_kernel<3><<<T.n_target_boxes, kSplitThreads, 0, s>>>(A);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? VL1_OK : cuda_fail(e, "split_remainder_kernel launch");
}
