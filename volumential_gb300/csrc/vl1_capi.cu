// C ABI of the list-1 evaluator: plan lifetime, status word, error strings.
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <mutex>
#include <new>

#include "vl1_internal.cuh"

namespace vl1 {

static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int32_t cuda_fail(cudaError_t e, const char *what) {
  set_error("%s: %s", what, cudaGetErrorString(e));
  return VL1_E_CUDA;
}

// The library's stream-ordered allocations (plans, schedule builders, table
// build scratch) come from a memory pool of its own in which memory freed on
// one stream is reused by another only once the free has completed: the
// device's default pool would instead make the allocating stream wait for
// the freeing stream's pending work, so that a plan admitted while a table
// build runs on another stream waited for that build to finish.
cudaError_t lib_malloc_async(void **ptr, size_t bytes, cudaStream_t s) {
  constexpr int kMaxDevices = 64;
  static std::mutex mu;
  static cudaMemPool_t pools[kMaxDevices] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  cudaMemPool_t pool;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (!pools[dev]) {
      cudaMemPoolProps props;
      memset(&props, 0, sizeof(props));
      props.allocType = cudaMemAllocationTypePinned;
      props.handleTypes = cudaMemHandleTypeNone;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = dev;
      cudaMemPool_t created = nullptr;
      e = cudaMemPoolCreate(&created, &props);
      if (e != cudaSuccess) return e;
      int off = 0;
      uint64_t keep = 1ull << 30;   // bytes kept cached across synchronisations
      e = cudaMemPoolSetAttribute(created, cudaMemPoolReuseAllowInternalDependencies, &off);
      if (e == cudaSuccess)
        e = cudaMemPoolSetAttribute(created, cudaMemPoolAttrReleaseThreshold, &keep);
      if (e != cudaSuccess) {
        cudaMemPoolDestroy(created);
        return e;
      }
      pools[dev] = created;
    }
    pool = pools[dev];
  }
  return cudaMallocFromPoolAsync(ptr, bytes, pool, s);
}

}  // namespace vl1

using namespace vl1;

namespace {

int32_t plan_alloc(vl1_plan *p, void **out, size_t bytes) {
  if (p->n_allocs >= (int)(sizeof(p->allocs) / sizeof(p->allocs[0]))) {
    set_error("internal: too many plan allocations");
    return VL1_E_NOMEM;
  }
  // stream-ordered allocation on the legacy stream: unlike cudaMalloc /
  // cudaFree it never waits for work on other streams (a serving engine
  // admits plans while table builds run on a stream of their own)
  void *ptr = nullptr;
  cudaError_t e = lib_malloc_async(&ptr, bytes ? bytes : 16, 0);
  if (e != cudaSuccess) {
    set_error("stream-ordered allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    return VL1_E_NOMEM;
  }
  p->allocs[p->n_allocs++] = ptr;
  p->device_bytes += (int64_t)bytes;
  *out = ptr;
  return VL1_OK;
}

template <typename T>
int32_t upload(vl1_plan *p, const T **dev, const void *host, size_t bytes) {
  void *ptr = nullptr;
  int32_t st = plan_alloc(p, &ptr, bytes);
  if (st) return st;
  if (bytes) {
    cudaError_t e = cudaMemcpy(ptr, host, bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(plan upload)");
  }
  *dev = static_cast<const T *>(ptr);
  return VL1_OK;
}

// the plan's device memory is freed in the order of `s`
void free_plan(vl1_plan *p, cudaStream_t s) {
  for (int i = 0; i < p->n_allocs; ++i) cudaFreeAsync(p->allocs[i], s);
  p->n_allocs = 0;
  delete p;
}

}  // namespace

extern "C" {

int32_t vl1_version(void) { return 100; }

const char *vl1_last_error_string(void) { return g_err; }

int32_t vl1_plan_create(const vl1_plan_desc *desc, vl1_plan **plan_out) {
  if (!desc || !plan_out) {
    set_error("vl1_plan_create: null argument");
    return VL1_E_ARG;
  }
  *plan_out = nullptr;
  if (desc->dim != 2 && desc->dim != 3) {
    set_error("arithmetic orbit reconstruction supports dim 2 or 3, got %d", desc->dim);
    return VL1_E_UNSUPPORTED;
  }
  if (desc->reconstruction_kind != VL1_RECON_SCALAR_ARITH &&
      desc->reconstruction_kind != VL1_RECON_SIGNED_ARITH &&
      desc->reconstruction_kind != VL1_RECON_DENSE) {
    set_error("unsupported reconstruction kind %d: the scalar/signed arithmetic orbit "
              "reconstruction and the dense table have device paths",
              desc->reconstruction_kind);
    return VL1_E_UNSUPPORTED_RECON;
  }
  const bool dense = desc->reconstruction_kind == VL1_RECON_DENSE;
  if (desc->quad_order < 1 || desc->n_tables < 1 || desc->n_table_entries < 1 ||
      desc->n_cases < 1 || desc->n_case_codes < 1 || !desc->table_data ||
      !desc->mode_nmlz || !desc->case_indices ||
      (!dense && (desc->n_case_orbits < 1 || !desc->case_orbit_ranks ||
                  !desc->case_axis_perm || !desc->case_axis_sign ||
                  !desc->case_axis_group || !desc->case_value_offsets ||
                  !desc->axis_sign_power || !desc->axis_direction_signs))) {
    set_error("vl1_plan_create: invalid plan description");
    return VL1_E_ARG;
  }
  int64_t nq = 1;
  for (int i = 0; i < desc->dim; ++i) nq *= desc->quad_order;
  if (nq > 1024) {
    set_error("q^dim = %lld exceeds the supported 1024 points per box", (long long)nq);
    return VL1_E_UNSUPPORTED;
  }
  if (dense && (int64_t)desc->n_table_entries != (int64_t)desc->n_cases * nq * nq) {
    set_error("a dense table has n_cases * n_q_points^2 = %lld entries per level, not %d",
              (long long)desc->n_cases * nq * nq, desc->n_table_entries);
    return VL1_E_ARG;
  }
  if (desc->value_type != VL1_REAL64 && desc->value_type != VL1_COMPLEX128) {
    set_error("value_type must be VL1_REAL64 or VL1_COMPLEX128");
    return VL1_E_ARG;
  }
  if (desc->displacement_kind == VL1_DISP_LOG2D && desc->dim != 2) {
    set_error("the log displacement is defined for 2D kernels only");
    return VL1_E_ARG;
  }

  vl1_plan *p = new (std::nothrow) vl1_plan();
  if (!p) {
    set_error("host allocation failed");
    return VL1_E_NOMEM;
  }
  memset(p, 0, sizeof(*p));
  cudaGetDevice(&p->device);

  DevDesc &d = p->d;
  d.dim = desc->dim;
  d.q = desc->quad_order;
  d.nq = (int)nq;
  d.n_tables = desc->n_tables;
  d.n_entries = desc->n_table_entries;
  d.n_cases = desc->n_cases;
  d.n_orbits = dense ? 0 : desc->n_case_orbits;
  d.n_case_codes = desc->n_case_codes;
  d.encoding_base = desc->encoding_base;
  d.direction_sign_axis = desc->direction_sign_axis;
  d.table_cplx = desc->value_type == VL1_COMPLEX128;
  d.scaling_exponent = desc->scaling_exponent;
  d.disp_kind = desc->displacement_kind;
  d.level_kind = desc->table_level_kind;
  d.table_starting_level = desc->table_starting_level;
  d.encoding_shift = desc->encoding_shift;
  d.bias = desc->case_encoding_bias;
  d.disp_coef = desc->displacement_coef;
  d.table_root_extent = desc->table_root_extent;

  const size_t vsz = d.table_cplx ? 16 : 8;
  const size_t dim = (size_t)d.dim;
  int32_t st = VL1_OK;
  if (!st) st = upload(p, &d.table, desc->table_data, vsz * d.n_tables * (size_t)d.n_entries);
  if (!st) st = upload(p, &d.nmlz, desc->mode_nmlz, vsz * d.n_tables * (size_t)nq);
  if (!st) st = upload(p, &d.case_indices, desc->case_indices, 8 * (size_t)d.n_case_codes);
  if (!dense) {
    if (!st) st = upload(p, &d.orbit_ranks, desc->case_orbit_ranks, 2 * (size_t)d.n_cases);
    if (!st) st = upload(p, &d.perm, desc->case_axis_perm, dim * d.n_cases);
    if (!st) st = upload(p, &d.sign, desc->case_axis_sign, dim * d.n_cases);
    if (!st) st = upload(p, &d.group, desc->case_axis_group, dim * d.n_cases);
    if (!st) st = upload(p, &d.offsets, desc->case_value_offsets, 4 * (size_t)(d.n_orbits + 1));
    if (!st) st = upload(p, &d.sign_power, desc->axis_sign_power, dim);
    if (!st) st = upload(p, &d.dir_signs, desc->axis_direction_signs, dim);
  }
  if (!st) {
    void *ptr = nullptr;
    st = plan_alloc(p, &ptr, sizeof(vl1_status));
    if (!st) {
      p->status = static_cast<vl1_status *>(ptr);
      cudaError_t e = cudaMemset(ptr, 0, sizeof(vl1_status));
      if (e != cudaSuccess) st = cuda_fail(e, "cudaMemset(status)");
    }
  }
  if (!st && !dense) {
    // Validate the descriptor offsets on the host: every row the arithmetic
    // can produce must lie inside the table.
    const int32_t *off = desc->case_value_offsets;
    if (off[0] != 0 || off[d.n_orbits] > d.n_entries) {
      set_error("case_value_offsets end at %d but the table has %d entries",
                off[d.n_orbits], d.n_entries);
      st = VL1_E_ENTRY_OOB;
    }
    for (int c = 0; !st && c < d.n_cases; ++c)
      if (desc->case_orbit_ranks[c] >= d.n_orbits) {
        set_error("case_orbit_ranks[%d] = %d out of range", c, desc->case_orbit_ranks[c]);
        st = VL1_E_ARG;
      }
    for (int i = 0; !st && i < d.n_cases * d.dim; ++i)
      if (desc->case_axis_perm[i] >= d.dim || desc->case_axis_group[i] >= d.dim) {
        set_error("case axis descriptor %d out of range", i);
        st = VL1_E_ARG;
      }
  }
  if (!st) {
    p->block_elems = (int64_t)d.n_tables * d.n_cases * nq * nq;
    if (p->block_elems * (d.table_cplx ? 2 : 1) >= ((int64_t)1 << 31)) {
      set_error("expanded blocks (%lld values) exceed the 2^31 index range",
                (long long)p->block_elems);
      cudaStreamSynchronize(0);
      free_plan(p, 0);
      return VL1_E_UNSUPPORTED;
    }
    if (dense) {
      // the table is already laid out as the blocks [level][case][source][target]
      d.blocks = d.table;
    } else {
      void *ptr = nullptr;
      st = plan_alloc(p, &ptr, vsz * (size_t)p->block_elems);
      if (!st) {
        d.blocks = static_cast<const double *>(ptr);
        st = launch_expand_blocks(p, 0);
      }
    }
  }
  if (!st) {
    // tensor-core digit operands of the blocks
    const MixedGeom g = mixed_geometry(d.nq, d.table_cplx);
    p->mixed.geom = g;
    const int64_t elems = (int64_t)d.n_tables * d.n_cases * g.n_kc * kDigits * (int64_t)g.np * g.kc;
    void *ptr = nullptr;
    st = plan_alloc(p, &ptr, 2 * (size_t)elems);
    if (!st) {
      p->mixed.adig = static_cast<__half *>(ptr);
      p->mixed.adig_alloc = p->n_allocs - 1;
      p->mixed.adig_elems = elems;
      double amax = 0.0;
      const double *tv = static_cast<const double *>(desc->table_data);
      const int64_t ntv = (int64_t)d.n_tables * d.n_entries * (d.table_cplx ? 2 : 1);
      for (int64_t i = 0; i < ntv; ++i) amax = fmax(amax, fabs(tv[i]));
      if (!(amax < 1e300)) {
        set_error("table data contains non-finite values");
        st = VL1_E_NONFINITE;
      } else {
        st = build_mixed_operands(p, amax, 0);
      }
    }
  }
  if (!st) {
    // the plan's own work (uploads, block expansion, digit operands) was
    // ordered on the legacy stream; work on other streams is not waited for
    cudaError_t e = cudaStreamSynchronize(0);
    if (e != cudaSuccess) st = cuda_fail(e, "plan block expansion");
  }
  if (!st) {
    vl1_status hs;
    cudaError_t e = cudaMemcpy(&hs, p->status, sizeof(hs), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
      st = cuda_fail(e, "plan status read");
    } else if (hs.code != VL1_OK) {
      set_error("orbit descriptors produce %d rows outside the table (first case %d, row %d)",
                hs.count, hs.detail0, hs.detail1);
      st = hs.code;
    }
  }
  if (st) {
    cudaStreamSynchronize(0);
    free_plan(p, 0);
    return st;
  }
  *plan_out = p;
  return VL1_OK;
}

int32_t vl1_plan_destroy(vl1_plan *plan) {
  if (!plan) return VL1_OK;
  cudaDeviceSynchronize();
  free_plan(plan, 0);
  return VL1_OK;
}

int32_t vl1_plan_release(vl1_plan *plan, void *stream) {
  if (!plan) return VL1_OK;
  free_plan(plan, static_cast<cudaStream_t>(stream));
  return VL1_OK;
}

int64_t vl1_plan_device_bytes(const vl1_plan *plan) {
  return plan ? plan->device_bytes : 0;
}

}  // extern "C"

int32_t vl1::make_tree(const vl1_plan *plan, const vl1_tree_view *t, TreeDev &tr) {
  if (!t || t->n_target_boxes < 0) {
    set_error("invalid tree view");
    return VL1_E_ARG;
  }
  if (t->n_target_boxes > 0 &&
      (!t->target_boxes || !t->neighbor_source_boxes_starts ||
       !t->neighbor_source_boxes_lists || !t->box_centers || !t->box_levels ||
       !t->box_source_starts || !t->box_source_counts_nonchild ||
       !t->box_target_starts || !t->box_target_counts_nonchild ||
       !t->source_mode_ids || !t->target_point_ids)) {
    set_error("tree view has a null array");
    return VL1_E_ARG;
  }
  (void)plan;
  tr.n_tgt_boxes = t->n_target_boxes;
  tr.target_boxes = t->target_boxes;
  tr.starts = t->neighbor_source_boxes_starts;
  tr.lists = t->neighbor_source_boxes_lists;
  tr.aligned_nboxes = t->aligned_nboxes;
  tr.centers = t->box_centers;
  tr.levels = t->box_levels;
  tr.src_starts = t->box_source_starts;
  tr.src_counts = t->box_source_counts_nonchild;
  tr.tgt_starts = t->box_target_starts;
  tr.tgt_counts = t->box_target_counts_nonchild;
  tr.smode = t->source_mode_ids;
  tr.tmode = t->target_point_ids;
  tr.n_particles = t->n_particles;
  tr.nboxes = t->nboxes;
  tr.root_extent = t->root_extent;
  // same operation sequence as level_extent / pair_scaling on the device
  // (products and quotients only, so no contraction can change the rounding)
  for (int l = 0; l < kScaleLevels; ++l) {
    const double ext = t->root_extent * (1.0 / (double)(1LL << l));
    const int sp = plan->d.scaling_exponent;
    if (sp == 0) {
      tr.level_scale[l] = 1.0;
      continue;
    }
    const int n = sp > 0 ? sp : -sp;
    double num = ext, den = plan->d.table_root_extent;
    for (int k = 1; k < n; ++k) {
      num = num * ext;
      den = den * plan->d.table_root_extent;
    }
    tr.level_scale[l] = sp > 0 ? num / den : den / num;
  }
  for (int l = 0; l < kScaleLevels; ++l) {
    int ex = 0;
    const double fr = frexp(tr.level_scale[l], &ex);
    // 0.5 * 2^ex: a power of two within the normal range
    tr.level_scale_log2[l] =
        (fr == 0.5 && ex - 1 >= -120 && ex - 1 <= 120) ? (int8_t)(ex - 1) : (int8_t)kNoScaleLog2;
  }
  return VL1_OK;
}

extern "C" {

int32_t vl1_eval_fp64(vl1_plan *plan, const vl1_tree_view *tree, const void *coefs,
                      int32_t coef_type, int32_t nrhs, void *result, void *stream) {
  if (!plan) {
    set_error("vl1_eval_fp64: null plan");
    return VL1_E_ARG;
  }
  if (nrhs < 1 || (coef_type != VL1_REAL64 && coef_type != VL1_COMPLEX128)) {
    set_error("vl1_eval_fp64: nrhs must be >= 1 and coef_type REAL64/COMPLEX128");
    return VL1_E_ARG;
  }
  TreeDev tr;
  int32_t st = make_tree(plan, tree, tr);
  if (st) return st;
  if (tr.n_tgt_boxes == 0) return VL1_OK;
  if (!coefs || !result) {
    set_error("vl1_eval_fp64: null coefficient or result pointer");
    return VL1_E_ARG;
  }
  return launch_plain(plan, tr, static_cast<const double *>(coefs),
                      coef_type == VL1_COMPLEX128, nrhs, static_cast<double *>(result),
                      static_cast<cudaStream_t>(stream));
}

int32_t vl1_classify_pairs(vl1_plan *plan, const vl1_tree_view *tree, int32_t *keys,
                           void *stream) {
  if (!plan || !keys) {
    set_error("vl1_classify_pairs: null argument");
    return VL1_E_ARG;
  }
  TreeDev tr;
  int32_t st = make_tree(plan, tree, tr);
  if (st) return st;
  if (tr.n_tgt_boxes == 0) return VL1_OK;
  return launch_classify(plan, tr, keys, static_cast<cudaStream_t>(stream));
}

int64_t vl1_mixed_workspace_bytes(const vl1_plan *plan, const vl1_tree_view *tree,
                                  int32_t nrhs) {
  if (!plan || !tree || nrhs < 1) return -1;
  return mixed_workspace_bytes(plan, tree->nboxes, tree->n_target_boxes, nrhs);
}

int32_t vl1_plan_set_mixed_geometry(vl1_plan *plan, int32_t kc, int32_t nch) {
  if (!plan || (kc != 16 && kc != 32) || (nch != 16 && nch != 32 && nch != 64)) {
    set_error("vl1_plan_set_mixed_geometry: null plan, K chunk not 16 or 32 or column "
              "chunk not 16, 32 or 64");
    return VL1_E_ARG;
  }
  const DevDesc &d = plan->d;
  const MixedGeom g = mixed_geometry(d.nq, d.table_cplx, kc, nch);
  if (g.kc > g.kp) {
    set_error("vl1_plan_set_mixed_geometry: K chunk %d above the %d padded source points",
              kc, g.kp);
    return VL1_E_ARG;
  }
  const MixedGeom &o = plan->mixed.geom;
  if (g.kc == o.kc && g.nch == o.nch && g.np == o.np && g.kp == o.kp) return VL1_OK;
  const int64_t elems =
      (int64_t)d.n_tables * d.n_cases * g.n_kc * kDigits * (int64_t)g.np * g.kc;
  // no evaluation may be in flight: the old operands are released
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(e, "vl1_plan_set_mixed_geometry: synchronise");
  void *ptr = nullptr;
  e = lib_malloc_async(&ptr, 2 * (size_t)elems, 0);
  if (e != cudaSuccess) return cuda_fail(e, "allocation of the plan digit operands");
  const int k = plan->mixed.adig_alloc;
  cudaFreeAsync(plan->allocs[k], 0);
  plan->allocs[k] = ptr;
  plan->device_bytes += 2 * (elems - plan->mixed.adig_elems);
  plan->mixed.adig = static_cast<__half *>(ptr);
  plan->mixed.adig_elems = elems;
  plan->mixed.geom = g;
  int32_t st = build_mixed_operands(plan, plan->mixed.table_absmax, 0);
  if (st) return st;
  e = cudaDeviceSynchronize();
  return e == cudaSuccess ? VL1_OK : cuda_fail(e, "vl1_plan_set_mixed_geometry: rebuild");
}

int32_t vl1_mixed_geometry(const vl1_plan *plan, int32_t *out5) {
  if (!plan || !out5) {
    set_error("vl1_mixed_geometry: null argument");
    return VL1_E_ARG;
  }
  const MixedGeom &g = plan->mixed.geom;
  out5[0] = g.kp;
  out5[1] = g.kc;
  out5[2] = g.n_kc;
  out5[3] = g.np;
  out5[4] = g.nch;
  return VL1_OK;
}

int32_t vl1_eval_mixed(vl1_plan *plan, const vl1_tree_view *tree,
                       const vl1_mixed_schedule *schedule, const double *coefs,
                       int32_t nrhs, void *result, void *workspace,
                       int64_t workspace_bytes, void *stream) {
  if (!plan || !schedule || nrhs < 1) {
    set_error("vl1_eval_mixed: null plan/schedule or nrhs < 1");
    return VL1_E_ARG;
  }
  TreeDev tr;
  int32_t st = make_tree(plan, tree, tr);
  if (st) return st;
  if (tr.n_tgt_boxes == 0) return VL1_OK;
  if (!coefs || !result || tr.nboxes < 1 || schedule->n_tiles < 0 ||
      (schedule->n_tiles > 0 && (!schedule->tile_rows || !schedule->tile_key_start ||
                                 !schedule->key_ids || !schedule->key_xrow))) {
    set_error("vl1_eval_mixed: invalid coefficients, result, nboxes or schedule");
    return VL1_E_ARG;
  }
  if (reinterpret_cast<uintptr_t>(schedule->key_xrow) % 16 != 0) {
    set_error("vl1_eval_mixed: schedule key_xrow must be 16-byte aligned");
    return VL1_E_ARG;
  }
  if (schedule->n_items < 0 || (schedule->n_items > 0 && !schedule->items) ||
      schedule->n_splits < 0 || schedule->n_slots < 0 ||
      (schedule->n_splits > 0 &&
       (!schedule->split_counters || !schedule->split_partials || schedule->n_slots < 2 ||
        reinterpret_cast<uintptr_t>(schedule->split_partials) % 16 != 0))) {
    set_error("vl1_eval_mixed: invalid work items or split scratch in the schedule");
    return VL1_E_ARG;
  }
  return launch_mixed(plan, tr, tr.nboxes, *schedule, coefs, nrhs,
                      static_cast<double *>(result), workspace, workspace_bytes,
                      static_cast<cudaStream_t>(stream));
}

int32_t vl1_orbit_index_map(vl1_plan *plan, int32_t *rows, int8_t *signs, void *stream) {
  if (!plan || !rows || !signs) {
    set_error("vl1_orbit_index_map: null argument");
    return VL1_E_ARG;
  }
  if (plan->d.n_orbits == 0) {
    set_error("vl1_orbit_index_map: a dense-table plan has no orbit map");
    return VL1_E_UNSUPPORTED_RECON;
  }
  return launch_index_map(plan, rows, signs, static_cast<cudaStream_t>(stream));
}

int32_t vl1_status_read(vl1_plan *plan, vl1_status *out, int32_t reset, void *stream) {
  if (!plan || !out) {
    set_error("vl1_status_read: null argument");
    return VL1_E_ARG;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemcpyAsync(out, plan->status, sizeof(vl1_status),
                                  cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && reset)
    e = cudaMemsetAsync(plan->status, 0, sizeof(vl1_status), s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "vl1_status_read");
  return VL1_OK;
}

}  // extern "C"
