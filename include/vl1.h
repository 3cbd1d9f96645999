/*
 * vl1 -- list-1 near-field evaluation on GB300 (sm_103a), C ABI.
 *
 * Drop-in boundary for volumential's list-1 evaluator.  The reference runs one
 * loopy-generated OpenCL kernel, ``near_field``, from
 * ``NearFieldFromCSR.__call__`` (volumential/list1.py:1260-1487; kernel body
 * list1.py:1050-1200).  The Python package ``volumential_gb300`` keeps the
 * reference's class and argument names and calls the entry points below
 * through ctypes.  All array pointers in ``vl1_tree_view`` and the coefficient
 * / result pointers are DEVICE pointers owned by the caller; the plan owns the
 * table, the normalizers and the orbit descriptors (uploaded once per table
 * set, like the reference's payload cache, expansion_wrangler_fpnd.py:2939-3158).
 * Every call is ordered on the given CUDA stream and returns without a host
 * synchronisation; device-side validation writes a status word that
 * ``vl1_status_read`` returns.  No entry point throws, traps or aborts.
 */
#ifndef VL1_H
#define VL1_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The Python layer maps them to the reference's exceptions. */
enum {
  VL1_OK = 0,
  VL1_E_INVALID_CASE = 1,      /* case code outside the gallery (case_indices == -1);
                                  the reference reads out of bounds here */
  VL1_E_ENTRY_OOB = 2,         /* reconstructed row outside the table */
  VL1_E_LAYOUT = 3,            /* box count > q^dim or mode id out of range
                                  (expansion_wrangler_fpnd.py:427-463) */
  VL1_E_LEVEL = 4,             /* table level outside [0, n_tables) */
  VL1_E_NONFINITE = 5,         /* non-finite output (volume_fmm.py:991-995) */
  VL1_E_UNSUPPORTED_RECON = 6, /* reconstruction kind other than arithmetic orbit
                                  (list1.py:903-1048 generated/dense fallbacks) */
  VL1_E_TIMEOUT = 7,           /* a bounded device wait gave up */
  VL1_E_CUDA = 8,              /* a CUDA runtime call failed */
  VL1_E_ARG = 9,               /* invalid argument */
  VL1_E_NOMEM = 10,            /* device allocation failed */
  VL1_E_UNSUPPORTED = 11       /* configuration not supported by this build */
};

enum { VL1_REAL64 = 0, VL1_COMPLEX128 = 1 };
/* VL1_RECON_DENSE: table_data holds every entry of every level,
 * [n_tables][n_cases][n_q_points (source mode)][n_q_points (target point)]
 * (n_table_entries = n_cases * n_q_points^2), used as is; the case_* / axis_*
 * orbit arrays are not read (list1.py:1018-1048, the dense fallback for
 * kernels without an arithmetic orbit reconstruction). */
enum { VL1_RECON_SCALAR_ARITH = 0, VL1_RECON_SIGNED_ARITH = 1, VL1_RECON_DENSE = 2 };
enum { VL1_DISP_NONE = 0, VL1_DISP_LOG2D = 1 };
enum { VL1_LEVEL_ZERO = 0, VL1_LEVEL_PER_LEVEL = 1 };

typedef struct vl1_plan vl1_plan;

/* Table payload and kernel policy of one NearFieldFromCSR instance.
 * Replaces the payload dict of expansion_wrangler_fpnd.py:3129-3158 and the
 * table_data_shapes / policy strings of list1.py:91-207, 361-437.
 * All pointers are HOST pointers; vl1_plan_create copies them. */
typedef struct {
  int32_t dim;                 /* 2 or 3 */
  int32_t quad_order;          /* q, n_q_points = q^dim */
  int32_t n_tables;            /* table levels */
  int32_t n_table_entries;     /* compact rows per level */
  int32_t n_cases;             /* 33 (2D) or 139 (3D) */
  int32_t n_case_orbits;       /* canonical cases */
  int32_t value_type;          /* VL1_REAL64 or VL1_COMPLEX128 (table + normalizers) */
  int32_t reconstruction_kind; /* VL1_RECON_* */
  const void *table_data;      /* [n_tables][n_table_entries] */
  const void *mode_nmlz;       /* [n_tables][n_q_points] */
  const int64_t *case_indices; /* [n_case_codes], -1 where no case */
  int32_t n_case_codes;        /* encoding_base^dim */
  int32_t encoding_base;       /* 13 */
  double encoding_shift;       /* 6 */
  double case_encoding_bias;   /* 1e-10 (list1.py:46) */
  const uint16_t *case_orbit_ranks;  /* [n_cases] */
  const uint8_t *case_axis_perm;     /* [n_cases][dim] */
  const int8_t *case_axis_sign;      /* [n_cases][dim] */
  const uint8_t *case_axis_group;    /* [n_cases][dim] */
  const int32_t *case_value_offsets; /* [n_case_orbits + 1] */
  const uint8_t *axis_sign_power;    /* [dim] */
  const int8_t *axis_direction_signs;/* [dim] */
  int32_t direction_sign_axis;       /* -1 when no directional derivative */
  int32_t scaling_exponent;    /* scaling = (sbox_extent/table_root_extent)^p */
  int32_t displacement_kind;   /* VL1_DISP_* */
  double displacement_coef;    /* -0.5/pi for the 2D Laplace log term */
  int32_t table_level_kind;    /* VL1_LEVEL_* */
  double table_root_extent;
  int32_t table_starting_level;
} vl1_plan_desc;

/* Tree arrays of one call (list1.py:1264-1354 keyword arguments).
 * DEVICE pointers, caller owned. */
typedef struct {
  int32_t n_target_boxes;
  const int32_t *target_boxes;                 /* [n_target_boxes] */
  const int32_t *neighbor_source_boxes_starts; /* [n_target_boxes + 1] */
  const int32_t *neighbor_source_boxes_lists;  /* [nnz] */
  int64_t aligned_nboxes;                      /* stride of box_centers */
  const double *box_centers;                   /* [dim][aligned_nboxes] */
  const uint8_t *box_levels;                   /* [nboxes] */
  const int32_t *box_source_starts;
  const int32_t *box_source_counts_nonchild;
  const int32_t *box_target_starts;
  const int32_t *box_target_counts_nonchild;
  const int32_t *source_mode_ids;              /* [n_particles] */
  const int32_t *target_point_ids;             /* [n_particles] */
  int64_t n_particles;
  int64_t nboxes;                              /* length of box_levels */
  double root_extent;
} vl1_tree_view;

/* One CTA's share of the mixed-precision work: keys [key_begin, key_end) of
 * one tile (indices into key_ids / key_xrow, inside the tile's own range).
 * A tile with many keys is split into `nparts` items (part 0 .. nparts-1);
 * each adds its exact int64 partial sums into the slot of part 0 (slot -
 * part), and the item that finishes last writes the tile's results and
 * clears the slot.  Unsplit items have split = -1, part = 0, nparts = 1,
 * slot = -1. */
typedef struct {
  int32_t tile;
  int32_t key_begin;
  int32_t key_end;
  int32_t split;       /* index of the split tile (its counters), or -1 */
  int32_t part;
  int32_t nparts;
  int32_t slot;        /* partial-sum slot, or -1 */
  int32_t reserved;
} vl1_mixed_item;

/* Work schedule of the mixed-precision path for one tree and rhs count
 * (built by the host from vl1_classify_pairs).  A tile is 128 rows, each row
 * one (target box index j, rhs r) item encoded j * nrhs + r (-1 = empty row).
 * Tile t covers keys key_ids[tile_key_start[t] .. tile_key_start[t+1]); a key is
 * table_level * n_cases + case.  key_xrow[k * 128 + row] is the density row
 * (source box S, rhs r) encoded S * nrhs + r, or -1 when the row's target box
 * has no list-1 pair of that key.
 * items: n_items work items, launched in this order (longest first balances
 * the GPU); n_items == 0 means one item per tile covering all its keys.
 * split_counters: n_splits * n_chunks * 16 int32 (the counter of split tile
 * s and column chunk c at index (s * n_chunks + c) * 16), zero before the
 * first call; every call leaves them zero.  split_partials: n_slots * (128 * padded
 * output columns) * 8 bytes for split tiles (the parts of a split tile add
 * their exact int64 sums into the slot of its part 0), zero before the first
 * call; every call leaves it zero.  n_chunks: the
 * plan's output column chunks (padded output columns / columns per CTA) when
 * the split scratch was sized; a call on a plan with another count is
 * refused (VL1_E_ARG).
 * DEVICE pointers, caller owned; key_xrow 16-byte aligned. */
typedef struct {
  int32_t n_tiles;
  const int32_t *tile_rows;
  const int32_t *tile_key_start;
  const int32_t *key_ids;
  const int32_t *key_xrow;
  int32_t n_items;
  const vl1_mixed_item *items;
  int32_t n_splits;
  int32_t n_slots;
  int32_t *split_counters;
  void *split_partials;
  int32_t n_chunks;
} vl1_mixed_schedule;

typedef struct {
  int32_t code;        /* first error code seen since the last reset */
  int32_t count;       /* number of faulting items */
  int32_t detail0;     /* e.g. the target box of the first fault */
  int32_t detail1;     /* e.g. the list position of the first fault */
} vl1_status;

/* Library version (major*10000 + minor*100 + patch). */
int32_t vl1_version(void);

/* Human-readable message of the last error of the calling host thread. */
const char *vl1_last_error_string(void);

/* Upload the table payload and build the expanded per-case blocks.
 * Replaces _get_cached_nearfield_payload (expansion_wrangler_fpnd.py:2939-3158)
 * plus the per-pair RECONSTRUCT_ENTRY work of list1.py:604-854, which the
 * plan performs once per (table level, case, source mode, target point). */
int32_t vl1_plan_create(const vl1_plan_desc *desc, vl1_plan **plan_out);
/* Waits for the device to be idle, then frees the plan. */
int32_t vl1_plan_destroy(vl1_plan *plan);
/* Frees the plan without a device-wide synchronisation: its device memory
 * is released in the order of `stream` (stream-ordered allocator), so the
 * caller guarantees that every call using the plan was issued on `stream` or
 * has completed.  No reference counterpart (the reference's payload cache
 * lives as long as its wrangler); a serving engine evicting idle plans while
 * table builds run on another stream uses it. */
int32_t vl1_plan_release(vl1_plan *plan, void *stream);

/* Plain FP64 list-1 evaluation (the reference's near_field kernel,
 * list1.py:1050-1159, potential_kind=1) for nrhs right-hand sides.
 * coefs:  [nrhs][n_particles] of coef_type (VL1_REAL64 or VL1_COMPLEX128)
 * result: [nrhs][n_particles], complex128 if the table or the coefficients are
 *         complex, else float64; overwritten (not accumulated), like
 *         result[target_id] = sum(...) in list1.py:1137.
 * stream: a cudaStream_t (NULL = legacy default stream). */
int32_t vl1_eval_fp64(vl1_plan *plan, const vl1_tree_view *tree,
                      const void *coefs, int32_t coef_type, int32_t nrhs,
                      void *result, void *stream);

/* Table key (table_level * n_cases + case) of every list-1 pair, computed with
 * the reference's FP64 case encoding (list1.py:439-459, 1084-1091) and table
 * level rule (list1.py:361-437); keys: device array [nnz], -1 for pairs whose
 * case code is outside the gallery (also reported in the status word). */
int32_t vl1_classify_pairs(vl1_plan *plan, const vl1_tree_view *tree, int32_t *keys,
                           void *stream);

/* Schedule of the mixed path built on the device (no reference counterpart:
 * the reference recomputes every pair's case in its kernel and has no
 * schedule; this replaces the host pass a first call on a new tree would
 * otherwise wait for).  begin: classifies every list-1 pair with the
 * reference's case encoding (list1.py:439-459, 1084-1091), checks that each
 * box's source mode ids are distinct and in range, orders the target boxes by
 * key signature (rarest keys most significant; a stable radix sort) and sizes
 * the tiles of 128 rows, longest first; it synchronises the stream twice and
 * allocates its own scratch.  nnz: the length of neighbor_source_boxes_lists.
 * key_start: copies the tile key starts [n_tiles + 1] to host memory.
 * fill: writes the arrays of vl1_mixed_schedule into caller-owned device
 * memory: tile_rows [n_tiles * 128], tile_key_start [n_tiles + 1], key_ids
 * [n_entries], key_xrow [n_entries * 128] (16-byte aligned).  Errors: a pair
 * whose case is outside the gallery (VL1_E_INVALID_CASE), two source boxes of
 * one target box with the same key (VL1_E_ARG), a source mode id out of range
 * or repeated in a box (VL1_E_LAYOUT). */
typedef struct vl1_schedule_builder vl1_schedule_builder;
typedef struct {
  int32_t n_tiles;
  int64_t n_entries;
} vl1_schedule_sizes;
int32_t vl1_schedule_build_begin(vl1_plan *plan, const vl1_tree_view *tree, int64_t nnz,
                                 int32_t nrhs, vl1_schedule_builder **out,
                                 vl1_schedule_sizes *sizes, void *stream);
int32_t vl1_schedule_build_key_start(const vl1_schedule_builder *builder,
                                     int32_t *key_start_host);
int32_t vl1_schedule_build_fill(vl1_schedule_builder *builder, int32_t *tile_rows,
                                int32_t *tile_key_start, int32_t *key_ids, int32_t *key_xrow,
                                void *stream);
int32_t vl1_schedule_builder_destroy(vl1_schedule_builder *builder);

/* Work items of a mixed-path schedule (host code, no device access; no
 * reference counterpart).  Tiles with more keys than a cap are split into
 * nearly equal key ranges; items are ordered longest first (ties keep tile
 * order).  cap > 0: that cap; cap <= 0: the cap among 13 fractions of one
 * SM's share of all keys whose modelled finish time on n_sm one-CTA-per-SM
 * slots is shortest (per item 4 keys of start-up and drain, a split part 1.5
 * more, the last part of a split tile 2 more).  key_start: host
 * [n_tiles + 1]; items: host [capacity]; *n_items receives the count also
 * when the capacity is too small (VL1_E_ARG). */
int32_t vl1_mixed_work_items(const int32_t *key_start, int32_t n_tiles, int32_t cap,
                             int32_t n_sm, vl1_mixed_item *items, int32_t capacity,
                             int32_t *n_items, int32_t *n_splits, int32_t *n_slots);

/* Bytes of caller-provided device workspace vl1_eval_mixed needs. */
int64_t vl1_mixed_workspace_bytes(const vl1_plan *plan, const vl1_tree_view *tree,
                                  int32_t nrhs);

/* Operand geometry of the mixed path: out[0..4] = padded source points, K
 * chunk, K chunks, padded output columns, output columns per CTA. */
int32_t vl1_mixed_geometry(const vl1_plan *plan, int32_t *out5);

/* Tile shape of the plan's tensor-core kernel (no reference counterpart; the
 * reference's tuning point is its kernel choice, list1.py:1240-1258): K chunk
 * kc (16 or 32 source points per pipeline unit) and output columns per CTA
 * nch (16, 32 or 64).  Rebuilds the plan's digit operands; synchronises the
 * device, so no evaluation with the plan may be in flight.  Schedules are
 * tied to the column chunk count (vl1_mixed_schedule.n_chunks). */
int32_t vl1_plan_set_mixed_geometry(vl1_plan *plan, int32_t kc, int32_t nch);

/* Mixed-precision list-1 evaluation on the tensor cores: the same sum as
 * vl1_eval_fp64 (list1.py:1050-1159) computed from exact FP16 digit products:
 * table values and scaled densities as 5 balanced base-256 digits of a
 * 39-bit fixed-point form (the table against one power-of-two scale per
 * plan, the densities against one per right-hand side), exact FP32 partial
 * sums of digit products, exact int64 sums and one rounding to FP64; each
 * output's error is a few 2^-39 of (largest |table value|) x (largest
 * |scaled density| of its rhs) x (its number of source points).
 * coefs: real [nrhs][n_particles] float64; result as in vl1_eval_fp64.
 * workspace: caller-provided device memory of vl1_mixed_workspace_bytes. */
int32_t vl1_eval_mixed(vl1_plan *plan, const vl1_tree_view *tree,
                       const vl1_mixed_schedule *schedule, const double *coefs,
                       int32_t nrhs, void *result, void *workspace,
                       int64_t workspace_bytes, void *stream);

/* ---- Batches: many problems in one persistent launch -------------------
 * A batch is a fixed set of problems (different trees, depths, q, rhs
 * counts and plans) whose tensor-core evaluations run together: batched
 * preparation kernels, then one persistent launch per kernel shape (column
 * chunk width x K chunk) in which every CTA takes the next (problem, tile,
 * column chunk) work item from a queue, longest first.  vl1_batch_create
 * copies the schedules' work lists to the host, builds the combined list
 * and allocates one device buffer (parameters, work list, per-problem
 * workspaces); vl1_batch_eval then only enqueues memsets and kernels on
 * `stream` (no allocation, no host synchronisation), so its calls can be
 * recorded in a CUDA graph and replayed.  All pointers of the problems
 * (tree arrays, schedules, coefficients, results) are device pointers that
 * must stay valid and fixed for the life of the batch; every eval reads the
 * current coefficients and overwrites the results.  Replaces the separate
 * vl1_eval_mixed calls a caller would make per problem
 * (expansion_wrangler_fpnd.py:3417-3442 per output kernel and tree). */
typedef struct vl1_batch vl1_batch;

typedef struct {
  vl1_plan *plan;
  const vl1_tree_view *tree;
  const vl1_mixed_schedule *schedule;   /* built for this tree and nrhs */
  const double *coefs;                  /* [nrhs][n_particles], device */
  int32_t nrhs;
  void *result;                         /* as for vl1_eval_mixed, device */
  const vl1_mixed_item *host_items;     /* optional host copy of schedule->items
                                           (NULL: copied from the device) */
} vl1_batch_problem;

typedef struct {
  int32_t ctas_per_launch;   /* persistent CTAs per kernel shape; 0: one per SM */
  int64_t capacity_bytes;    /* device buffer of at least this size, so that
                                later vl1_batch_update calls fit (0: exact) */
} vl1_batch_options;

/* Two problems of one batch must not share a schedule that splits tiles
 * (its split scratch): give each problem its own schedule instance. */
int32_t vl1_batch_create(int32_t n_problems, const vl1_batch_problem *problems,
                         const vl1_batch_options *options, vl1_batch **out);
/* Replace the batch's problems (continuous batching: one call per serving
 * step).  No device allocation: the new parameters, work list and
 * workspaces must fit the batch's buffer (VL1_E_ARG otherwise); they are
 * assembled on the host (from host_items where given) and uploaded with one
 * asynchronous copy on `stream` from pinned staging owned by the batch.
 * The next vl1_batch_eval must be ordered after it on the same stream; an
 * update may wait (on the host) for the upload of the update before last.
 * CUDA graphs recorded before an update replay the old problem set's
 * launch shapes and must be recorded again. */
int32_t vl1_batch_update(vl1_batch *batch, int32_t n_problems,
                         const vl1_batch_problem *problems, void *stream);
int32_t vl1_batch_eval(vl1_batch *batch, void *stream);
int32_t vl1_batch_destroy(vl1_batch *batch);
/* Device bytes held by the batch (its own buffer; plans and schedules apart). */
int64_t vl1_batch_device_bytes(const vl1_batch *batch);
/* Kernels one vl1_batch_eval launches (preparation and tensor-core launches;
 * its one memset not counted). */
int32_t vl1_batch_kernel_launches(const vl1_batch *batch);

/* ---- Table builder: FP64 Duffy radial quadrature ----------------------
 * Values of near-field table entries, T = int_{[0,h]^d} G(t - y) phi(y) dy,
 * by the scheme of the reference's batched builder
 * (volumential/nearfield_potential_table.py:2035-2223, nodes :2225-2291;
 * 1D rules volumential/singular_integral_2d.py:807-853): the box split at
 * the clipped target into 2^d sub-boxes and d! Duffy simplices each, a
 * tanh-sinh radial rule and a Gauss-Legendre tail rule.  G includes the
 * kernel's scaling constant: Laplace 2D -log(r)/(2 pi), 3D 1/(4 pi r);
 * Helmholtz 2D (i/4) H0^(1)(k r), 3D exp(i k r)/(4 pi r); constant 1;
 * plane wave cos(k d_0) (a test kernel); r^power and r^power log r (the
 * Helmholtz split mode's extra term tables, expansion_wrangler_fpnd.py:
 * 144-209, scaling constant 1).  All arrays are device arrays;
 * result is [n_entries] doubles, or [n_entries][2] (re, im) when
 * complex_output.  Replaces _batched_duffy_values_for_local_indices
 * (nearfield_potential_table.py:2331-2463). */
enum {
  VL1_DUFFY_LAPLACE2D = 0,
  VL1_DUFFY_LAPLACE3D = 1,
  VL1_DUFFY_HELMHOLTZ2D = 2,
  VL1_DUFFY_HELMHOLTZ3D = 3,
  VL1_DUFFY_CONSTANT = 4,
  VL1_DUFFY_PLANE_WAVE = 5,
  VL1_DUFFY_POWER = 6,        /* r^power, power >= 0 */
  VL1_DUFFY_POWER_LOG = 7     /* r^power log r, power >= 1 */
};

typedef struct {
  int32_t dim, q, n_entries;
  int32_t n_reg, n_rad;       /* 1D rule sizes */
  int32_t kernel;             /* VL1_DUFFY_* */
  int32_t complex_output;
  int32_t max_ctas;           /* 0: one CTA per (entry, Duffy sub-simplex); else at
                                 most this many CTAs, striding over them (a build
                                 that leaves most SMs to other work) */
  int32_t power;              /* VL1_DUFFY_POWER / _POWER_LOG: the power of r (<= 64) */
  int32_t derivative;         /* Laplace / Helmholtz only: 0 none, a + 1 the target
                                 derivative d/dt_a, -(a + 1) the source derivative
                                 d/dy_a (AxisTarget/SourceDerivative) */
  double extent;              /* source box [0, extent]^dim */
  double k;                   /* Helmholtz / plane-wave wave number */
  const double *target_points;          /* [dim][n_entries] */
  const double *decomposition_targets;  /* [dim][n_entries]: targets clipped to the box */
  const int32_t *mode_axes;             /* [dim][n_entries]: source mode index per axis */
  const double *regular_nodes, *regular_weights;   /* [n_reg] on [0, 1] */
  const double *radial_nodes, *radial_weights;     /* [n_rad] on (0, 1) */
  const double *interp_nodes;    /* [q]: 1D Gauss-Legendre nodes on [0, extent] */
  const double *interp_weights;  /* [q]: 1 / prod_{j != m} (x_m - x_j) */
} vl1_duffy_desc;

int32_t vl1_duffy_table(const vl1_duffy_desc *desc, double *result, void *stream);

/* ---- Helmholtz split correction ---------------------------------------
 * The split mode's list-1 remainder (volumential/expansion_wrangler_fpnd.py:
 * 3491-3836, series remainder kernel :212-332; for split orders above 1 the
 * host zeroes the coefficients of the terms the extra tables carry):
 *   result[t] = sum over list-1 source points s (s != t when exclude_self)
 *               of weights[s] * R(|x_t - x_s|),
 *   2D: R(r) = c0 + sum_{n=1..N} (a_n log r + b_n) r^{2n},
 *   3D: R(r) = sum_{n=1..N} c_n r^{n-1},
 * coefficients [2][N + 1][2] (re, im): row 0 = (c0, a_1..a_N) in 2D or
 * (unused, c_1..c_N) in 3D, row 1 = (unused, b_1..b_N).  Points are the tree's
 * sources = targets (tree order, [dim][n_points]); the result is complex
 * [n_points][2] and is overwritten for the target boxes' points.
 * flags: VL1_SPLIT_REAL_K when the wave number is real (the coefficients then
 * have its structure: 2D a_n real and Im b_n = -(pi/2) a_n; 3D c_n real for
 * even n and imaginary for odd n), which halves the series work. */
#define VL1_SPLIT_REAL_K 1
typedef struct {
  int32_t dim, n_points, n_terms, exclude_self, weights_complex, flags;
  const vl1_tree_view *tree;
  const double *points;
  const double *weights;
  const double *coefficients;
  double *result;
} vl1_split_desc;

int32_t vl1_split_correction(const vl1_split_desc *desc, void *stream);

/* ---- List-1 interaction lists on the device ----------------------------
 * For every leaf (target box, ascending box id), the sorted distinct leaves
 * touching it at its level, one level coarser or one level finer (boxtree's
 * list 1, used at volumential/volume_fmm.py:984-989), as CSR.  Boxes are
 * given by their level and integer coordinates at that level.  Needs
 * vl1_list1_csr_workspace_bytes(n_leaves) of device workspace and
 * lists_capacity >= the list-1 entry count (n_leaves x 110 always suffices in
 * 3D, x 30 in 2D); *nnz (host) receives the entry count.  Synchronises the
 * stream (the entry count is read back). */
typedef struct {
  int32_t dim, nboxes, n_leaves, max_level;
  const uint8_t *box_levels;    /* [nboxes] */
  const int32_t *box_coords;    /* [nboxes][dim] */
  const int32_t *leaf_boxes;    /* [n_leaves], ascending */
  int32_t *starts;              /* [n_leaves + 1] out */
  int32_t *lists;               /* [lists_capacity] out */
  int64_t lists_capacity;
  void *workspace;
  int64_t workspace_bytes;
} vl1_csr_desc;

int64_t vl1_list1_csr_workspace_bytes(int32_t n_leaves);
int32_t vl1_list1_csr(const vl1_csr_desc *desc, int64_t *nnz, void *stream);

/* ---- Box trees on the device -----------------------------------------
 * 2:1 level restriction of a set of leaves (volumential/
 * tree_interactive_build.py:202-432): a leaf at level L splits every leaf at
 * a level below L - 1 that contains one of its same-level neighbour
 * positions, until none does.  levels/coords: device arrays of `capacity`
 * leaves ([capacity] uint8, [capacity][dim] int32 integer coordinates at the
 * leaf's level), of which *n_leaves are set; on return they hold the
 * balanced leaves (in no particular order) and *n_leaves their count
 * (VL1_E_ARG when they need more than `capacity`).  Synchronises the stream
 * once per pass and allocates its own scratch. */
int32_t vl1_tree_balance(int32_t dim, int32_t *n_leaves, int32_t capacity, uint8_t *levels,
                         int32_t *coords, void *stream);

/* The particle tree of a set of leaves (the layout of
 * build_particle_tree_from_box_tree, tree_interactive_build.py:1274-1441):
 * boxes are the leaves and their ancestors, numbered level by level and
 * lexicographically by integer coordinates inside a level; every leaf holds
 * the q^dim tensor Gauss-Legendre nodes of its box (meshgrid "ij" order),
 * leaves in box order.  begin: leaf_levels / leaf_coords are device arrays
 * of n_leaves distinct leaves of one tree; root_vertex is a host [dim];
 * sizes3 receives (nboxes, aligned_nboxes = nboxes rounded up to 32,
 * max_level).  level_starts: host [max_level + 2] first box of each level.
 * fill: ref_nodes host [dim][q^dim] and ref_weights host [q^dim] (the
 * reference nodes on [-1, 1] and the products of their weights); device
 * outputs box_levels [nboxes], box_coords [nboxes][dim], box_centers
 * [dim][aligned_nboxes], box_is_leaf [nboxes], box_starts / box_counts
 * [nboxes] (q^dim per leaf, 0 otherwise), leaf_boxes [n_leaves], targets
 * [dim][n_leaves q^dim], weights [n_leaves q^dim] (weights of the reference
 * rule times (extent / 2)^dim).  Synchronises the stream. */
typedef struct vl1_tree_builder vl1_tree_builder;
int32_t vl1_tree_build_begin(int32_t dim, int32_t q, int32_t n_leaves, const uint8_t *leaf_levels,
                             const int32_t *leaf_coords, double root_extent,
                             const double *root_vertex, vl1_tree_builder **out,
                             int32_t *sizes3, void *stream);
int32_t vl1_tree_build_level_starts(const vl1_tree_builder *builder, int32_t *out);
int32_t vl1_tree_build_fill(vl1_tree_builder *builder, const double *ref_nodes,
                            const double *ref_weights, uint8_t *box_levels, int32_t *box_coords,
                            double *box_centers, uint8_t *box_is_leaf, int32_t *box_starts,
                            int32_t *box_counts, int32_t *leaf_boxes, double *targets,
                            double *weights, void *stream);
int32_t vl1_tree_builder_destroy(vl1_tree_builder *builder);

/* Measurement hook (no reference counterpart): while `begin` and `end` are
 * set (cudaEvent_t handles, or NULL to stop), every vl1_eval_mixed and
 * vl1_batch_eval records `begin` on its stream right before its tensor-core
 * kernel launch(es) and `end` right after, so that a caller can time that
 * kernel alone with cudaEventElapsedTime.  Process-wide; not for concurrent
 * callers. */
int32_t vl1_set_kernel_events(void *begin, void *end);

/* Test hook (no reference counterpart): every wait of the tensor-core kernel
 * on a pipeline barrier is bounded in time; a wait that runs out sets the
 * launch's abort flag, the kernel lets its issued copies and MMAs complete,
 * frees its TMEM, writes no results and reports VL1_E_TIMEOUT in the status
 * word.  wait_limit_us: microseconds before a wait gives up, 0 = the default
 * (2 s).  withhold_arrival != 0: in the next launches, one producer warp of
 * CTA (0, 0) does not signal its first pipeline unit, so that the issuer's
 * wait on it runs out (a barrier that nothing completes; no fault).
 * Process-wide; vl1_test_set_wait_fault(0, 0) restores normal operation.  A
 * schedule that timed out stays usable. */
int32_t vl1_test_set_wait_fault(int32_t wait_limit_us, int32_t withhold_arrival);

/* Size of the fixed scratch array used by vl1_eval_mixed_noalloc (32 MiB). */
#define VL1_NOALLOC_SCRATCH_BYTES (32LL << 20)

/* vl1_eval_mixed without caller-provided workspace, for callers that cannot
 * allocate device memory (a host code that owns all device memory through its
 * own pool and only hands over the arrays it computes on; a latency-critical
 * loop where cudaMalloc's device synchronisation or failure is not an option).
 * No counterpart in the reference: it has no device-side scratch to manage.
 * Same inputs and outputs as vl1_eval_mixed; the scratch lives in a fixed
 * VL1_NOALLOC_SCRATCH_BYTES array inside this library (held on every GPU that
 * loads the library, until the process exits).  Problems needing more scratch
 * than that (vl1_mixed_workspace_bytes) are rejected with VL1_E_ARG.  No
 * cudaMalloc, cudaFree or other allocating call is made.  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress) with that
 * device current, and a call looks it up again when the CUDA context current
 * on the device is not the one of the last lookup (the address is bound to
 * that context); make the first call in each context before any stream
 * capture.  All calls share the array: calls that overlap on the GPU race and
 * must be serialised by the caller.  The plan must belong to the current
 * device. */
int32_t vl1_eval_mixed_noalloc(vl1_plan *plan, const vl1_tree_view *tree,
                               const vl1_mixed_schedule *schedule, const double *coefs,
                               int32_t nrhs, void *result, void *stream);

/* Row and sign of every (table level 0, case, source mode, target point) as the
 * device computes them: rows/signs are device arrays [n_cases][nq][nq].
 * Exposes the integer index of list1.py:604-854 for bit-exact checks. */
int32_t vl1_orbit_index_map(vl1_plan *plan, int32_t *rows, int8_t *signs,
                            void *stream);

/* Copy the device status word to the host (synchronises the stream) and,
 * when reset != 0, clear it. */
int32_t vl1_status_read(vl1_plan *plan, vl1_status *out, int32_t reset,
                        void *stream);

/* Bytes of device memory the plan holds (tables, blocks, descriptors). */
int64_t vl1_plan_device_bytes(const vl1_plan *plan);

#ifdef __cplusplus
}
#endif

#endif /* VL1_H */
