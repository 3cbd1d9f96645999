/*
 * CPU oracle of the list-1 near-field evaluation -- TEST INFRASTRUCTURE.
 *
 * This file is a plain-C restatement of the reference's generated OpenCL
 * kernel ``near_field`` (volumential/list1.py:1050-1159) with the
 * scalar/signed arithmetic orbit reconstruction (volumential/list1.py:604-854).
 * It is used only by the tests, by ``__graft_entry__.smoke()`` and by the CPU
 * baseline legs of ``bench.py`` -- as the checker and as the timed stand-in
 * for the reference's pocl CPU path, never as part of the product.
 *
 * Mapping follows the reference: one OpenMP work item per target box (pocl
 * runs one work-group per target box, list1.py:1256), the per-pair case id,
 * scaling, displacement and orbit row recomputed for every (target point,
 * source point) pair, FP64 (or complex128) accumulation in (source box,
 * source point) order.
 *
 * Compile: cc -O2 -fopenmp -ffp-contract=off -fno-fast-math -shared -fPIC
 * (contraction off keeps every FP64 operation a separately rounded IEEE op).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define VL1O_OK 0
#define VL1O_E_INVALID_CASE 1
#define VL1O_E_ENTRY_OOB 2
#define VL1O_E_LAYOUT 3
#define VL1O_E_ARG 9

typedef struct {
  int32_t dim, q, n_tables, n_entries, n_cases;
  int32_t table_is_complex, coef_is_complex;
  const double *table_data; /* [n_tables][n_entries] (x2 interleaved if complex) */
  const double *mode_nmlz;  /* [n_tables][q^dim]     (x2 interleaved if complex) */
  const int64_t *case_indices;
  int32_t n_case_codes, encoding_base;
  double encoding_shift, case_encoding_bias;
  const uint16_t *case_orbit_ranks;
  const uint8_t *case_axis_perm;
  const int8_t *case_axis_sign;
  const uint8_t *case_axis_group;
  const int32_t *case_value_offsets;
  int32_t n_orbits;
  const uint8_t *axis_sign_power;
  const int8_t *axis_direction_signs;
  int32_t direction_sign_axis;
  /* scaling policy (volumential/list1.py:361-437) */
  int32_t scaling_exponent;     /* scaling = (ext/table_root_extent)^p, p may be <0 */
  int32_t displacement_kind;    /* 0: none, 1: 2D log displacement */
  double disp_coef;             /* -0.5/pi for 2D Laplace */
  int32_t table_level_per_level;/* 0: table level 0, 1: per-level selection */
  double root_extent, table_root_extent;
  int32_t table_starting_level;
} vl1o_params;

/* Compact row and sign of entry (case, source mode, target point), following
 * the generated reconstruction code of list1.py:604-854. */
int vl1o_orbit_row(const vl1o_params *p, int case_id, int source_mode_id,
                   int target_point_id, int32_t *row_out, int32_t *sign_out) {
  const int dim = p->dim, q = p->q;
  int src_raw[3], tgt_raw[3];
  if (dim == 2) {
    src_raw[0] = source_mode_id / q;
    src_raw[1] = source_mode_id % q;
    tgt_raw[0] = target_point_id / q;
    tgt_raw[1] = target_point_id % q;
  } else if (dim == 3) {
    src_raw[0] = source_mode_id / (q * q);
    src_raw[1] = (source_mode_id / q) % q;
    src_raw[2] = source_mode_id % q;
    tgt_raw[0] = target_point_id / (q * q);
    tgt_raw[1] = (target_point_id / q) % q;
    tgt_raw[2] = target_point_id % q;
  } else {
    return VL1O_E_ARG;
  }

  int src[3], tgt[3], group[3], axis_sign[3];
  int entry_sign = 1;
  for (int i = 0; i < dim; ++i) {
    int perm = p->case_axis_perm[case_id * dim + i];
    int sgn = p->case_axis_sign[case_id * dim + i];
    group[i] = p->case_axis_group[case_id * dim + i];
    axis_sign[i] = sgn;
    int sign_power = p->axis_sign_power[perm];
    int s_raw = src_raw[perm], t_raw = tgt_raw[perm];
    int s_fixed = sgn < 0 ? q - 1 - s_raw : s_raw;
    int t_fixed = sgn < 0 ? q - 1 - t_raw : t_raw;
    int s_flip = q - 1 - s_raw, t_flip = q - 1 - t_raw;
    int zero_flip = (sgn == 0 && (s_flip < s_raw || (s_flip == s_raw && t_flip < t_raw)));
    src[i] = zero_flip ? s_flip : s_fixed;
    tgt[i] = zero_flip ? t_flip : t_fixed;
    int transform_sign = (sgn < 0 || zero_flip) ? -1 : 1;
    int dir_factor = 1;
    if (p->direction_sign_axis == i)
      dir_factor = transform_sign * p->axis_direction_signs[perm] *
                   p->axis_direction_signs[i];
    entry_sign *= (sign_power != 0 ? transform_sign : 1) * dir_factor;
  }

  /* compare-exchange network over axes of equal group */
#define CSWAP(a, b)                                                          \
  do {                                                                       \
    if (group[a] == group[b] &&                                              \
        (src[b] < src[a] || (src[b] == src[a] && tgt[b] < tgt[a]))) {        \
      int ts = src[a]; src[a] = src[b]; src[b] = ts;                         \
      int tt = tgt[a]; tgt[a] = tgt[b]; tgt[b] = tt;                         \
    }                                                                        \
  } while (0)
  if (dim == 2) {
    CSWAP(0, 1);
  } else {
    CSWAP(0, 1);
    CSWAP(1, 2);
    CSWAP(0, 1);
    CSWAP(0, 2);
  }
#undef CSWAP

  int64_t pair[3];
  for (int i = 0; i < dim; ++i) pair[i] = (int64_t)src[i] * q + tgt[i];
  const int64_t pair_count = (int64_t)q * q;
  const int64_t folded = (pair_count + 1) / 2;

  int64_t rank_g[3], count_g[3];
  for (int g = 0; g < dim; ++g) {
    int size = 0, zeros = 0;
    int64_t lo = pair_count, hi = -1, sum = 0;
    for (int i = 0; i < dim; ++i) {
      if (group[i] != g) continue;
      ++size;
      if (axis_sign[i] == 0) ++zeros;
      if (pair[i] < lo) lo = pair[i];
      if (pair[i] > hi) hi = pair[i];
      sum += pair[i];
    }
    int64_t A = zeros > 0 ? folded : pair_count;
    int64_t mid = sum - lo - hi;
    if (size == 0) {
      count_g[g] = 1;
      rank_g[g] = 0;
    } else if (size == 1) {
      count_g[g] = A;
      rank_g[g] = lo;
    } else if (size == 2) {
      count_g[g] = A * (A + 1) / 2;
      rank_g[g] = A * (A + 1) / 2 - (A - lo) * (A - lo + 1) / 2 + (hi - lo);
    } else {
      count_g[g] = A * (A + 1) * (A + 2) / 6;
      rank_g[g] = A * (A + 1) * (A + 2) / 6 -
                  (A - lo) * (A - lo + 1) * (A - lo + 2) / 6 +
                  (A - lo) * (A - lo + 1) / 2 - (A - mid) * (A - mid + 1) / 2 +
                  (hi - mid);
    }
  }
  int64_t compact;
  if (dim == 2)
    compact = rank_g[0] * count_g[1] + rank_g[1];
  else
    compact = (rank_g[0] * count_g[1] + rank_g[1]) * count_g[2] + rank_g[2];
  int orbit = p->case_orbit_ranks[case_id];
  *row_out = (int32_t)(p->case_value_offsets[orbit] + compact);
  *sign_out = entry_sign;
  return VL1O_OK;
}

/* rows/signs of every (case, source mode, target point): [n_cases][nq][nq] */
int vl1o_full_map(const vl1o_params *p, int32_t *rows, int8_t *signs) {
  int nq = 1;
  for (int i = 0; i < p->dim; ++i) nq *= p->q;
  for (int c = 0; c < p->n_cases; ++c)
    for (int s = 0; s < nq; ++s)
      for (int t = 0; t < nq; ++t) {
        int32_t r, sg;
        int st = vl1o_orbit_row(p, c, s, t, &r, &sg);
        if (st) return st;
        size_t k = ((size_t)c * nq + s) * nq + t;
        rows[k] = r;
        signs[k] = (int8_t)sg;
      }
  return VL1O_OK;
}

static double ipow2_inv(int level) {
  /* 1.0 / (2**level) with an integer power, as the reference kernel does */
  int64_t d = (int64_t)1 << level;
  return 1.0 / (double)d;
}

/* result[target] for every target of every target box (list1.py:1060-1139).
 * coefs and result hold n_particles values (interleaved re/im if complex).
 * Returns the first error status seen (the reference would read out of
 * bounds in those cases; the oracle reports instead). */
int vl1o_near_field(const vl1o_params *p, int n_tgt_boxes,
                    const int32_t *target_boxes, const int32_t *nbr_starts,
                    const int32_t *nbr_lists, int64_t aligned_nboxes,
                    const double *box_centers, const uint8_t *box_levels,
                    const int32_t *box_source_starts,
                    const int32_t *box_source_counts,
                    const int32_t *box_target_starts,
                    const int32_t *box_target_counts,
                    const int32_t *source_mode_ids,
                    const int32_t *target_point_ids, const double *coefs,
                    double *result, int nthreads) {
  const int dim = p->dim;
  int nq = 1;
  for (int i = 0; i < dim; ++i) nq *= p->q;
  const int out_complex = p->table_is_complex || p->coef_is_complex;
  int status = VL1O_OK;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif

#pragma omp parallel for schedule(dynamic, 4)
  for (int tbox = 0; tbox < n_tgt_boxes; ++tbox) {
    const int target_box_id = target_boxes[tbox];
    const int box_target_beg = box_target_starts[target_box_id];
    const int n_box_targets = box_target_counts[target_box_id];
    const int sbox_begin = nbr_starts[tbox], sbox_end = nbr_starts[tbox + 1];
    int local_status = VL1O_OK;

    for (int tid = 0; tid < nq; ++tid) {
      if (tid >= n_box_targets) continue;
      const int target_id = box_target_beg + tid;
      const int target_point_id = target_point_ids[target_id];
      double acc_re = 0.0, acc_im = 0.0;

      for (int sbox = sbox_begin; sbox < sbox_end; ++sbox) {
        const int source_box_id = nbr_lists[sbox];
        const int n_box_sources = box_source_counts[source_box_id];
        const int box_source_beg = box_source_starts[source_box_id];
        const int sbox_level = box_levels[source_box_id];
        const double sbox_extent = p->root_extent * ipow2_inv(sbox_level);

        int table_lev = 0;
        if (p->table_level_per_level) {
          int d = sbox_level - p->table_starting_level;
          table_lev = sbox_level < p->table_starting_level
                          ? 0
                          : (d < p->n_tables ? d : p->n_tables - 1);
        }

        double vec = 0.0;
        for (int d = 0; d < dim; ++d) {
          double comp = (box_centers[d * aligned_nboxes + target_box_id] -
                         box_centers[d * aligned_nboxes + source_box_id]) /
                            sbox_extent * 4.0 +
                        p->encoding_shift + p->case_encoding_bias;
          vec = vec * (double)p->encoding_base + comp;
        }
        const int vec_id = (int)(vec + 0.5);
        if (vec_id < 0 || vec_id >= p->n_case_codes) {
          local_status = VL1O_E_INVALID_CASE;
          continue;
        }
        const int case_id = (int)p->case_indices[vec_id];
        if (case_id < 0 || case_id >= p->n_cases) {
          local_status = VL1O_E_INVALID_CASE;
          continue;
        }

        double scaling = 1.0;
        const int pe = p->scaling_exponent;
        if (pe != 0) {
          int n = pe > 0 ? pe : -pe;
          double num = sbox_extent, den = p->table_root_extent;
          for (int k = 1; k < n; ++k) {
            num = num * sbox_extent;
            den = den * p->table_root_extent;
          }
          scaling = pe > 0 ? num / den : den / num;
        }

        for (int sid = 0; sid < n_box_sources; ++sid) {
          const int source_id = box_source_beg + sid;
          const int source_mode_id = source_mode_ids[source_id];
          if (source_mode_id < 0 || source_mode_id >= nq || target_point_id < 0 ||
              target_point_id >= nq || sid >= nq) {
            local_status = VL1O_E_LAYOUT;
            continue;
          }
          int32_t entry_id, entry_sign;
          vl1o_orbit_row(p, case_id, source_mode_id, target_point_id, &entry_id,
                         &entry_sign);
          if (entry_id < 0 || entry_id >= p->n_entries) {
            local_status = VL1O_E_ENTRY_OOB;
            continue;
          }
          double t_re, t_im = 0.0, n_re = 0.0, n_im = 0.0;
          size_t ti = (size_t)table_lev * p->n_entries + entry_id;
          size_t ni = (size_t)table_lev * nq + sid;
          if (p->table_is_complex) {
            t_re = p->table_data[2 * ti];
            t_im = p->table_data[2 * ti + 1];
            if (p->displacement_kind) {
              n_re = p->mode_nmlz[2 * ni];
              n_im = p->mode_nmlz[2 * ni + 1];
            }
          } else {
            t_re = p->table_data[ti];
            if (p->displacement_kind) n_re = p->mode_nmlz[ni];
          }
          /* displacement = c * scaling * log(ext / table_root_extent) * nmlz */
          double disp_re = 0.0, disp_im = 0.0;
          if (p->displacement_kind == 1) {
            double f = p->disp_coef * scaling * log(sbox_extent / p->table_root_extent);
            disp_re = f * n_re;
            disp_im = f * n_im;
          }
          double integ_re = t_re * (double)entry_sign * scaling + disp_re;
          double integ_im = t_im * (double)entry_sign * scaling + disp_im;
          if (p->coef_is_complex) {
            double c_re = coefs[2 * source_id], c_im = coefs[2 * source_id + 1];
            acc_re = acc_re + (c_re * integ_re - c_im * integ_im);
            acc_im = acc_im + (c_re * integ_im + c_im * integ_re);
          } else {
            double c = coefs[source_id];
            acc_re = acc_re + c * integ_re;
            acc_im = acc_im + c * integ_im;
          }
        }
      }
      if (out_complex) {
        result[2 * target_id] = acc_re;
        result[2 * target_id + 1] = acc_im;
      } else {
        result[target_id] = acc_re;
      }
    }
    if (local_status != VL1O_OK) {
#pragma omp critical
      if (status == VL1O_OK) status = local_status;
    }
  }
  return status;
}

/* Case id and table level of every list-1 pair (target box position tbox,
 * list position k), computed with the expressions of the main loop above
 * (list1.py:1084-1091 case encoding, :1086-1087 / :361-437 table level).
 * case_ids[k] = -1 where the code falls outside the gallery. */
int vl1o_classify_pairs(const vl1o_params *p, int n_tgt_boxes, const int32_t *target_boxes,
                        const int32_t *nbr_starts, const int32_t *nbr_lists,
                        int64_t aligned_nboxes, const double *box_centers,
                        const uint8_t *box_levels, int32_t *case_ids,
                        int32_t *table_levels) {
  const int dim = p->dim;
  int status = VL1O_OK;
  for (int tbox = 0; tbox < n_tgt_boxes; ++tbox) {
    const int target_box_id = target_boxes[tbox];
    for (int k = nbr_starts[tbox]; k < nbr_starts[tbox + 1]; ++k) {
      const int source_box_id = nbr_lists[k];
      const int sbox_level = box_levels[source_box_id];
      const double sbox_extent = p->root_extent * ipow2_inv(sbox_level);
      int table_lev = 0;
      if (p->table_level_per_level) {
        int d = sbox_level - p->table_starting_level;
        table_lev = sbox_level < p->table_starting_level
                        ? 0
                        : (d < p->n_tables ? d : p->n_tables - 1);
      }
      double vec = 0.0;
      for (int d = 0; d < dim; ++d) {
        double comp = (box_centers[d * aligned_nboxes + target_box_id] -
                       box_centers[d * aligned_nboxes + source_box_id]) /
                          sbox_extent * 4.0 +
                      p->encoding_shift + p->case_encoding_bias;
        vec = vec * (double)p->encoding_base + comp;
      }
      const int vec_id = (int)(vec + 0.5);
      int case_id = -1;
      if (vec_id >= 0 && vec_id < p->n_case_codes) case_id = (int)p->case_indices[vec_id];
      if (case_id < 0 || case_id >= p->n_cases) {
        case_id = -1;
        status = VL1O_E_INVALID_CASE;
      }
      case_ids[k] = case_id;
      table_levels[k] = table_lev;
    }
  }
  return status;
}

/* Number of threads OpenMP would use (reported beside CPU timings). */
int vl1o_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
