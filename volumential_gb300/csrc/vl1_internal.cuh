// Internal declarations shared by the vl1 translation units (not installed).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "vl1.h"
#include "vl1_mixed.cuh"

namespace vl1 {

// Everything a kernel needs from the plan, passed by value.
struct DevDesc {
  int dim, q, nq;
  int n_tables, n_entries, n_cases, n_orbits;
  int n_case_codes, encoding_base, direction_sign_axis;
  int table_cplx;
  int scaling_exponent, disp_kind, level_kind, table_starting_level;
  double encoding_shift, bias, disp_coef, table_root_extent;
  const int64_t *case_indices;
  const uint16_t *orbit_ranks;
  const uint8_t *perm;
  const int8_t *sign;
  const uint8_t *group;
  const int32_t *offsets;
  const uint8_t *sign_power;
  const int8_t *dir_signs;
  const double *table;   // [n_tables][n_entries] (x2 complex)
  const double *nmlz;    // [n_tables][nq]        (x2 complex)
  const double *blocks;  // [n_tables][n_cases][nq(s)][nq(t)] (x2 complex)
};

// Tree view on the device side (copied from vl1_tree_view).
struct TreeDev {
  int n_tgt_boxes;
  const int32_t *target_boxes, *starts, *lists;
  int64_t aligned_nboxes;
  const double *centers;
  const uint8_t *levels;
  const int32_t *src_starts, *src_counts, *tgt_starts, *tgt_counts;
  const int32_t *smode, *tmode;
  int64_t n_particles;
  int64_t nboxes;
  double root_extent;
  // scaling of a source box of level l (l < kScaleLevels), computed on the
  // host with the same IEEE operations as pair_scaling(level_extent(l))
  double level_scale[32];
  // log2 of level_scale[l] when it is an exact power of two (a dyadic tree
  // and table extent), else kNoScaleLog2: the density planes then scale by
  // an exponent shift instead of an FP64 multiply
  int8_t level_scale_log2[32];
};
constexpr int kNoScaleLog2 = 127;
constexpr int kScaleLevels = 32;
constexpr int kTileRows = 128;   // rows (target box, rhs) of a mixed-path tile

}  // namespace vl1

struct vl1_plan {
  int device;
  vl1::DevDesc d;
  int64_t block_elems;  // n_tables * n_cases * nq * nq
  int64_t device_bytes;
  void *allocs[16];
  int n_allocs;
  vl1_status *status;   // device
  vl1::MixedPlan mixed;
};

namespace vl1 {

void set_error(const char *fmt, ...);
int32_t cuda_fail(cudaError_t e, const char *what);
// stream-ordered allocation from the library's own pool (vl1_capi.cu); free
// with cudaFreeAsync
cudaError_t lib_malloc_async(void **ptr, size_t bytes, cudaStream_t s);
// vl1_tree_view -> TreeDev with host validation (vl1_capi.cu)
int32_t make_tree(const vl1_plan *plan, const vl1_tree_view *t, TreeDev &tr);

// Launchers (stream-ordered, no host synchronisation).
int32_t launch_expand_blocks(vl1_plan *plan, cudaStream_t s);
int32_t launch_index_map(vl1_plan *plan, int32_t *rows, int8_t *signs, cudaStream_t s);
int32_t launch_plain(vl1_plan *plan, const TreeDev &tree, const double *coefs,
                     int coef_cplx, int nrhs, double *result, cudaStream_t s);
// operand geometry; kc / nch 0: the default choice (else 16 or 32 / 16, 32
// or 64, validated by the caller)
MixedGeom mixed_geometry(int nq, int table_cplx, int kc = 0, int nch = 0);
int32_t build_mixed_operands(vl1_plan *plan, double table_absmax, cudaStream_t s);
int64_t mixed_workspace_bytes(const vl1_plan *plan, int64_t nboxes, int64_t n_tgt_boxes,
                              int nrhs);
int32_t launch_classify(vl1_plan *plan, const TreeDev &tree, int32_t *keys, cudaStream_t s);
int32_t launch_mixed(vl1_plan *plan, const TreeDev &tree, int64_t nboxes,
                     const vl1_mixed_schedule &sched, const double *coefs, int nrhs,
                     double *result, void *workspace, int64_t ws_bytes, cudaStream_t s);

// ---------------------------------------------------------------------------
// Device helpers

__device__ __forceinline__ void report(vl1_status *st, int code, int d0, int d1) {
  if (atomicCAS(&st->code, 0, code) == 0) {
    st->detail0 = d0;
    st->detail1 = d1;
  }
  atomicAdd(&st->count, 1);
}

// Compact table row and sign of (case c, source mode s, target point t).
// Integer restatement of the arithmetic orbit reconstruction of
// volumential/list1.py:604-854: per output axis take the permuted input axis,
// reflect it (sign < 0) or fold it onto the lexicographically smaller of the
// pair and its reflection (sign == 0); sort axes of equal group with the fixed
// compare-exchange network; rank each group's sorted pair codes as a multiset
// in closed form; combine group ranks in mixed radix; add the case orbit's
// offset.  The sign is the product of the reflections on odd axes (and the
// directional-derivative line sign).
__device__ __forceinline__ void orbit_row(const DevDesc &d, int c, int s, int t,
                                          int &row, int &sign) {
  const int q = d.q, dim = d.dim;
  int sa[3], ta[3];
  if (dim == 2) {
    sa[0] = s / q; sa[1] = s - sa[0] * q;
    ta[0] = t / q; ta[1] = t - ta[0] * q;
  } else {
    const int q2 = q * q;
    sa[0] = s / q2; sa[1] = (s / q) % q; sa[2] = s % q;
    ta[0] = t / q2; ta[1] = (t / q) % q; ta[2] = t % q;
  }
  int src[3], tgt[3], grp[3], zs[3];
  int esign = 1;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    if (i >= dim) break;
    const int in = d.perm[c * dim + i];
    const int sg = d.sign[c * dim + i];
    grp[i] = d.group[c * dim + i];
    zs[i] = (sg == 0);
    const int s0 = sa[in], t0 = ta[in];
    const int s1 = q - 1 - s0, t1 = q - 1 - t0;
    const bool flip = (sg < 0) || (sg == 0 && (s1 < s0 || (s1 == s0 && t1 < t0)));
    src[i] = flip ? s1 : s0;
    tgt[i] = flip ? t1 : t0;
    const int ts = flip ? -1 : 1;
    if (d.sign_power[in]) esign *= ts;
    if (d.direction_sign_axis == i) esign *= ts * d.dir_signs[in] * d.dir_signs[i];
  }
  auto cswap = [&](int a, int b) {
    if (grp[a] == grp[b] && (src[b] < src[a] || (src[b] == src[a] && tgt[b] < tgt[a]))) {
      int x = src[a]; src[a] = src[b]; src[b] = x;
      x = tgt[a]; tgt[a] = tgt[b]; tgt[b] = x;
    }
  };
  if (dim == 2) {
    cswap(0, 1);
  } else {
    cswap(0, 1); cswap(1, 2); cswap(0, 1); cswap(0, 2);
  }
  const long long pc = (long long)q * q;
  const long long folded = (pc + 1) / 2;
  long long compact = 0;
  for (int g = 0; g < dim; ++g) {
    int n = 0, z = 0;
    long long lo = pc, hi = -1, sum = 0;
    for (int i = 0; i < dim; ++i) {
      if (grp[i] != g) continue;
      const long long pr = (long long)src[i] * q + tgt[i];
      ++n; z += zs[i];
      lo = pr < lo ? pr : lo;
      hi = pr > hi ? pr : hi;
      sum += pr;
    }
    const long long A = z ? folded : pc;
    long long cnt, rk;
    if (n == 0) {
      cnt = 1; rk = 0;
    } else if (n == 1) {
      cnt = A; rk = lo;
    } else if (n == 2) {
      cnt = A * (A + 1) / 2;
      rk = cnt - (A - lo) * (A - lo + 1) / 2 + (hi - lo);
    } else {
      const long long mid = sum - lo - hi;
      cnt = A * (A + 1) * (A + 2) / 6;
      rk = cnt - (A - lo) * (A - lo + 1) * (A - lo + 2) / 6 +
           (A - lo) * (A - lo + 1) / 2 - (A - mid) * (A - mid + 1) / 2 + (hi - mid);
    }
    compact = compact * cnt + rk;
  }
  row = (int)(d.offsets[d.orbit_ranks[c]] + compact);
  sign = esign;
}

// Case id of a (target box, source box) pair with the reference's FP64 case
// encoding (list1.py:439-459, 532-538, 1084, 1089-1091), every operation
// rounded separately so that the code is the one the reference computes.
// Returns -1 when the code is outside the gallery.
__device__ __forceinline__ int pair_case_id(const DevDesc &d, const TreeDev &tr,
                                            int tbox_id, int sbox_id,
                                            double sbox_extent) {
  double v = 0.0;
  for (int a = 0; a < d.dim; ++a) {
    const double ct = tr.centers[a * tr.aligned_nboxes + tbox_id];
    const double cs = tr.centers[a * tr.aligned_nboxes + sbox_id];
    double comp = __ddiv_rn(__dsub_rn(ct, cs), sbox_extent);
    comp = __dadd_rn(__dadd_rn(__dmul_rn(comp, 4.0), d.encoding_shift), d.bias);
    v = __dadd_rn(__dmul_rn(v, (double)d.encoding_base), comp);
  }
  const int code = __double2int_rz(__dadd_rn(v, 0.5));
  if (code < 0 || code >= d.n_case_codes) return -1;
  const long long c = d.case_indices[code];
  return (c < 0 || c >= d.n_cases) ? -1 : (int)c;
}

// sbox_extent = root_extent * (1.0 / 2**level)   (list1.py:1084)
__device__ __forceinline__ double level_extent(double root_extent, int level) {
  return __dmul_rn(root_extent, __ddiv_rn(1.0, (double)(1LL << level)));
}

// scaling = sbox_extent^p / table_root_extent^p, multiplied out left to right
// as the generated scaling code does (list1.py:295-313).
__device__ __forceinline__ double pair_scaling(const DevDesc &d, double ext) {
  const int p = d.scaling_exponent;
  if (p == 0) return 1.0;
  const int n = p > 0 ? p : -p;
  double num = ext, den = d.table_root_extent;
  for (int k = 1; k < n; ++k) {
    num = __dmul_rn(num, ext);
    den = __dmul_rn(den, d.table_root_extent);
  }
  return p > 0 ? __ddiv_rn(num, den) : __ddiv_rn(den, num);
}

// scaling of a source box of `level`: from the per-call table when the level
// is in it (the FP64 pipe is narrow on this GPU; the division chain of
// pair_scaling is then done once per level on the host)
__device__ __forceinline__ double box_scaling(const DevDesc &d, const TreeDev &tr, int level) {
  if (level < kScaleLevels) return tr.level_scale[level];
  return pair_scaling(d, level_extent(tr.root_extent, level));
}

// table level of a source box (list1.py:361-437, 1086-1087)
__device__ __forceinline__ int pair_table_level(const DevDesc &d, int level) {
  if (d.level_kind != VL1_LEVEL_PER_LEVEL) return 0;
  const int rel = level - d.table_starting_level;
  if (level < d.table_starting_level) return 0;
  return rel < d.n_tables ? rel : d.n_tables - 1;
}

}  // namespace vl1
