// Device-side build of the mixed path's tile schedule (vl1_schedule_build_*).
//
// The tensor-core kernel walks tiles of 128 (target box, rhs) rows and, per
// tile, the table keys (table level, case) its boxes use.  This builds that
// schedule from the tree on the device, so that a first call on a new tree
// does not wait for a host pass over the pairs:
//
//   1. one warp per target box classifies its list-1 pairs with the
//      reference's FP64 case encoding (the arithmetic of vl1_classify_pairs),
//      sets the box's key bits (a second source box with the same key is an
//      error) and counts how often each key occurs; one thread per box checks
//      that the box's source mode ids are distinct and in range;
//   2. (host, one synchronisation) keys are ranked by frequency, rarest
//      first;
//   3. every box gets a sort key: its key set as a bit string with the
//      rarest key most significant; a stable LSD radix sort (one pass per
//      64-bit word) orders the boxes, so boxes with equal key sets are
//      adjacent and tiles of consecutive rows share most of their keys;
//   4. the key union of every tile (tiles of 128 consecutive rows) and its
//      size; (host, one synchronisation) tiles are ordered longest first;
//   5. the arrays of vl1_mixed_schedule: tile rows, per-tile key lists in
//      ascending key order, and the density row of every (tile key, row).
//
// The result has the layout and the meaning of the host builder's schedule;
// only the order of the boxes (which decides how well tiles share keys)
// differs from the host's greedy packing.
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "vl1_internal.cuh"

namespace vl1 {
namespace {

constexpr int kSchedOk = 0;
constexpr int kSchedDuplicateKey = 1;   // two source boxes of one target box share a key
constexpr int kSchedInvalidCase = 2;    // a pair's case code is outside the gallery
constexpr int kSchedModeRange = 3;      // a source mode id outside [0, q^dim)
constexpr int kSchedModeDuplicate = 4;  // two sources of one box share a mode id
constexpr int kSchedBadNnz = 5;         // the CSR's last start is not nnz

struct SchedStatus {
  int code;
  int detail0, detail1;
};

__device__ __forceinline__ void sched_report(SchedStatus *st, int code, int d0, int d1) {
  if (atomicCAS(&st->code, 0, code) == 0) {
    st->detail0 = d0;
    st->detail1 = d1;
  }
}

// Step 1: classify the pairs of each target box (one warp per box).
__global__ void sched_classify_kernel(DevDesc d, TreeDev tr, int64_t nnz, int words,
                                      int32_t *keys, int32_t *pair_box,
                                      unsigned long long *box_mask, int32_t *freq,
                                      SchedStatus *st) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  if (blockIdx.x == 0 && threadIdx.x == 0 && tr.n_tgt_boxes > 0 &&
      tr.starts[tr.n_tgt_boxes] != nnz)
    sched_report(st, kSchedBadNnz, tr.starts[tr.n_tgt_boxes], (int)nnz);
  for (int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; i < tr.n_tgt_boxes;
       i += warps) {
    const int tbox = tr.target_boxes[i];
    const int p0 = tr.starts[i], p1 = tr.starts[i + 1];
    for (int p = p0 + lane; p < p1; p += 32) {
      if (p < 0 || p >= nnz) continue;
      const int sbox = tr.lists[p];
      const int lvl = tr.levels[sbox];
      const int c = pair_case_id(d, tr, tbox, sbox, level_extent(tr.root_extent, lvl));
      int key = -1;
      if (c < 0) {
        sched_report(st, kSchedInvalidCase, (int)i, p);
      } else {
        key = pair_table_level(d, lvl) * d.n_cases + c;
        const unsigned long long bit = 1ull << (key & 63);
        const unsigned long long old =
            atomicOr(box_mask + i * words + (key >> 6), bit);
        if (old & bit) sched_report(st, kSchedDuplicateKey, (int)i, key);
        atomicAdd(freq + key, 1);
      }
      keys[p] = key;
      pair_box[p] = (int32_t)i;
    }
  }
}

// Step 1b: source mode ids of every box with sources distinct and in range
// (the mixed path places every source point at its mode's column).
__global__ void sched_check_modes_kernel(TreeDev tr, int nq, SchedStatus *st) {
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < tr.nboxes;
       b += (int64_t)gridDim.x * blockDim.x) {
    const int cnt = tr.src_counts[b];
    if (cnt <= 0) continue;
    const int s0 = tr.src_starts[b];
    unsigned seen[32];   // nq <= 1024
    for (int w = 0; w < 32; ++w) seen[w] = 0u;
    const int n = cnt < nq ? cnt : nq;
    for (int s = 0; s < n; ++s) {
      const int m = tr.smode[s0 + s];
      if (m < 0 || m >= nq) {
        sched_report(st, kSchedModeRange, (int)b, s);
        break;
      }
      if (seen[m >> 5] & (1u << (m & 31))) {
        sched_report(st, kSchedModeDuplicate, (int)b, m);
        break;
      }
      seen[m >> 5] |= 1u << (m & 31);
    }
  }
}

// Step 3a: the sort key of every box: bit (63 - rank % 64) of word rank / 64
// for each of its keys, rank = the key's place in the rarest-first order.
__global__ void sched_sort_key_kernel(int n_tb, int words, const unsigned long long *box_mask,
                                      const int32_t *rank, unsigned long long *sort_key) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_tb;
       i += (int64_t)gridDim.x * blockDim.x) {
    unsigned long long *out = sort_key + i * words;
    for (int w = 0; w < words; ++w) out[w] = 0ull;
    for (int w = 0; w < words; ++w) {
      unsigned long long m = box_mask[i * words + w];
      while (m) {
        const int b = __ffsll((long long)m) - 1;
        m &= m - 1;
        const int r = rank[w * 64 + b];
        out[r >> 6] |= 1ull << (63 - (r & 63));
      }
    }
  }
}

__global__ void sched_gather_word_kernel(int n_tb, int words, int w,
                                         const unsigned long long *sort_key,
                                         const int32_t *order, unsigned long long *out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_tb;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = sort_key[(int64_t)order[i] * words + w];
}

__global__ void sched_iota_kernel(int n, int32_t *out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (int32_t)i;
}

__global__ void sched_inverse_kernel(int n, const int32_t *order, int32_t *pos) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    pos[order[i]] = (int32_t)i;
}

// Step 4: key union of every tile (a box's rows may span several tiles).
__global__ void sched_tile_mask_kernel(int n_tb, int words, int nrhs,
                                       const unsigned long long *box_mask, const int32_t *pos,
                                       unsigned long long *tile_mask) {
  const int64_t n = (int64_t)n_tb * words;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx / words;
    const int w = (int)(idx - i * words);
    const unsigned long long m = box_mask[idx];
    if (!m) continue;
    const int64_t r0 = (int64_t)pos[i] * nrhs, r1 = r0 + nrhs - 1;
    for (int64_t t = r0 / kTileRows; t <= r1 / kTileRows; ++t)
      atomicOr(tile_mask + t * words + w, m);
  }
}

__global__ void sched_tile_count_kernel(int n_tiles, int words,
                                        const unsigned long long *tile_mask, int32_t *counts) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n_tiles;
       t += (int64_t)gridDim.x * blockDim.x) {
    int c = 0;
    for (int w = 0; w < words; ++w) c += __popcll(tile_mask[t * words + w]);
    counts[t] = c;
  }
}

// Step 5: schedule arrays (tiles in the longest-first order lpt).
__global__ void sched_tile_rows_kernel(int n_tiles, int64_t n_rows, int nrhs,
                                       const int32_t *lpt, const int32_t *order,
                                       int32_t *tile_rows) {
  const int64_t n = (int64_t)n_tiles * kTileRows;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = idx / kTileRows, j = idx - t * kTileRows;
    const int64_t row = (int64_t)lpt[t] * kTileRows + j;
    int32_t v = -1;
    if (row < n_rows) v = (int32_t)((int64_t)order[row / nrhs] * nrhs + row % nrhs);
    tile_rows[idx] = v;
  }
}

__global__ void sched_key_ids_kernel(int n_tiles, int words, const int32_t *lpt,
                                     const unsigned long long *tile_mask,
                                     const int32_t *key_start, int32_t *key_ids) {
  const int64_t n = (int64_t)n_tiles * words;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = idx / words;
    const int w = (int)(idx - t * words);
    const unsigned long long *m = tile_mask + (int64_t)lpt[t] * words;
    int base = key_start[t];
    for (int v = 0; v < w; ++v) base += __popcll(m[v]);
    unsigned long long x = m[w];
    while (x) {
      const int b = __ffsll((long long)x) - 1;
      x &= x - 1;
      key_ids[base++] = w * 64 + b;
    }
  }
}

__global__ void sched_xrow_kernel(int64_t nnz, int nrhs, int words, const int32_t *keys,
                                  const int32_t *pair_box, const int32_t *lists,
                                  const int32_t *pos, const int32_t *inv_lpt,
                                  const int32_t *key_start,
                                  const unsigned long long *tile_mask, int32_t *xrow) {
  const int64_t n = nnz * nrhs;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = idx / nrhs;
    const int r = (int)(idx - p * nrhs);
    const int key = keys[p];
    if (key < 0) continue;
    const int64_t row = (int64_t)pos[pair_box[p]] * nrhs + r;
    const int64_t t = row / kTileRows;
    const unsigned long long *m = tile_mask + t * words;
    int rank = 0;
    for (int v = 0; v < (key >> 6); ++v) rank += __popcll(m[v]);
    rank += __popcll(m[key >> 6] & ((1ull << (key & 63)) - 1ull));
    const int64_t entry = (int64_t)key_start[inv_lpt[t]] + rank;
    xrow[entry * kTileRows + (row - t * kTileRows)] =
        (int32_t)((int64_t)lists[p] * nrhs + r);
  }
}

int grid1d(int64_t n, int threads) {
  int64_t g = (n + threads - 1) / threads;
  if (g > 152 * 16) g = 152 * 16;
  return (int)(g < 1 ? 1 : g);
}

int64_t align256(int64_t b) { return (b + 255) / 256 * 256; }

}  // namespace
}  // namespace vl1

struct vl1_schedule_builder {
  int device = -1;
  vl1::TreeDev tree;
  int n_tb = 0, nrhs = 1, n_keys = 0, words = 1;
  int64_t nnz = 0, n_rows = 0;
  int n_tiles = 0;
  int64_t n_entries = 0;
  void *buf = nullptr;   // one device allocation for all scratch
  cudaStream_t stream = nullptr;   // the builder's stream (its scratch is freed there)
  int32_t *keys = nullptr, *pair_box = nullptr, *freq = nullptr, *rank = nullptr;
  unsigned long long *box_mask = nullptr, *sort_key = nullptr, *word_a = nullptr,
                     *word_b = nullptr, *tile_mask = nullptr;
  int32_t *order_a = nullptr, *order_b = nullptr, *pos = nullptr, *counts = nullptr;
  int32_t *lpt = nullptr, *inv_lpt = nullptr, *key_start = nullptr;
  void *cub_tmp = nullptr;
  size_t cub_bytes = 0;
  vl1::SchedStatus *status = nullptr;
  std::vector<int32_t> host_key_start;   // [n_tiles + 1], longest-first order
};

using namespace vl1;

namespace {

int32_t sched_status_error(const SchedStatus &s) {
  switch (s.code) {
    case kSchedOk:
      return VL1_OK;
    case kSchedDuplicateKey:
      set_error("a target box has two list-1 source boxes with the same case (target box "
                "index %d, key %d)", s.detail0, s.detail1);
      return VL1_E_ARG;
    case kSchedInvalidCase:
      set_error("list1 case encoding produced codes outside the interaction gallery (first "
                "at target box index %d, list position %d); the tree is not 2:1 balanced "
                "or box centres are inconsistent", s.detail0, s.detail1);
      return VL1_E_INVALID_CASE;
    case kSchedModeRange:
      set_error("source mode id outside [0, q^dim) in box %d (source %d)", s.detail0,
                s.detail1);
      return VL1_E_LAYOUT;
    case kSchedModeDuplicate:
      set_error("duplicate source mode ids inside box %d (mode %d)", s.detail0, s.detail1);
      return VL1_E_LAYOUT;
    case kSchedBadNnz:
      set_error("neighbor_source_boxes_starts ends at %d, not at the list length %d",
                s.detail0, s.detail1);
      return VL1_E_ARG;
    default:
      set_error("schedule build: status %d", s.code);
      return VL1_E_ARG;
  }
}

}  // namespace

namespace {

int32_t schedule_begin(vl1_plan *plan, const vl1_tree_view *tree, int64_t nnz, int32_t nrhs,
                       vl1_schedule_builder *b, vl1_schedule_sizes *sizes, cudaStream_t s);

}  // namespace

extern "C" int32_t vl1_schedule_build_begin(vl1_plan *plan, const vl1_tree_view *tree,
                                            int64_t nnz, int32_t nrhs,
                                            vl1_schedule_builder **out,
                                            vl1_schedule_sizes *sizes, void *stream) {
  if (!plan || !tree || !out || !sizes || nrhs < 1 || nnz < 0) {
    set_error("vl1_schedule_build_begin: null argument, nrhs < 1 or nnz < 0");
    return VL1_E_ARG;
  }
  *out = nullptr;
  vl1_schedule_builder *b = new vl1_schedule_builder();
  const int32_t st = schedule_begin(plan, tree, nnz, nrhs, b, sizes,
                                    static_cast<cudaStream_t>(stream));
  if (st != VL1_OK) {
    // the scratch is released in stream order, after the launched work
    if (b->buf) cudaFreeAsync(b->buf, static_cast<cudaStream_t>(stream));
    delete b;
    return st;
  }
  *out = b;
  return VL1_OK;
}

namespace {

int32_t schedule_begin(vl1_plan *plan, const vl1_tree_view *tree, int64_t nnz, int32_t nrhs,
                       vl1_schedule_builder *b, vl1_schedule_sizes *sizes, cudaStream_t s) {
  if (plan->d.nq > 1024) {
    set_error("vl1_schedule_build_begin: q^dim = %d above 1024", plan->d.nq);
    return VL1_E_UNSUPPORTED;
  }
  int32_t st = make_tree(plan, tree, b->tree);
  if (st) return st;
  cudaGetDevice(&b->device);
  b->n_tb = b->tree.n_tgt_boxes;
  b->nrhs = nrhs;
  b->n_keys = plan->d.n_tables * plan->d.n_cases;
  b->words = (b->n_keys + 63) / 64;
  b->nnz = nnz;
  b->n_rows = (int64_t)b->n_tb * nrhs;
  if (b->n_rows / kTileRows >= INT32_MAX || nnz >= INT32_MAX) {
    set_error("vl1_schedule_build_begin: %lld rows / %lld pairs exceed 32-bit indices",
              (long long)b->n_rows, (long long)nnz);
    return VL1_E_UNSUPPORTED;
  }
  b->n_tiles = (int)((b->n_rows + kTileRows - 1) / kTileRows);
  const int W = b->words, K = b->n_keys, n = b->n_tb, T = b->n_tiles;

  // scratch: one allocation, carved in 256-byte aligned pieces
  size_t cub_bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, cub_bytes, (unsigned long long *)nullptr,
                                  (unsigned long long *)nullptr, (int32_t *)nullptr,
                                  (int32_t *)nullptr, n > 0 ? n : 1, 0, 64, s);
  const int64_t sz[] = {
      align256(4 * std::max<int64_t>(nnz, 1)),            // keys
      align256(4 * std::max<int64_t>(nnz, 1)),            // pair_box
      align256(4 * (int64_t)K),                           // freq
      align256(4 * (int64_t)K),                           // rank
      align256(8 * (int64_t)n * W),                       // box_mask
      align256(8 * (int64_t)n * W),                       // sort_key
      align256(8 * (int64_t)std::max(n, 1)),              // word_a
      align256(8 * (int64_t)std::max(n, 1)),              // word_b
      align256(8 * (int64_t)std::max(T, 1) * W),          // tile_mask
      align256(4 * (int64_t)std::max(n, 1)),              // order_a
      align256(4 * (int64_t)std::max(n, 1)),              // order_b
      align256(4 * (int64_t)std::max(n, 1)),              // pos
      align256(4 * (int64_t)std::max(T, 1)),              // counts
      align256(4 * (int64_t)std::max(T, 1)),              // lpt
      align256(4 * (int64_t)std::max(T, 1)),              // inv_lpt
      align256(4 * ((int64_t)T + 1)),                     // key_start
      align256((int64_t)cub_bytes),                       // cub scratch
      align256(sizeof(SchedStatus))};
  int64_t total = 0;
  for (int64_t v : sz) total += v;
  // stream-ordered: never waits for work on other streams
  cudaError_t e = lib_malloc_async(&b->buf, total, s);
  if (e != cudaSuccess) {
    b->buf = nullptr;
    return cuda_fail(e, "allocation of the schedule builder scratch");
  }
  b->stream = s;
  uint8_t *p = static_cast<uint8_t *>(b->buf);
  int k = 0;
  auto take = [&](auto *&ptr) {
    ptr = reinterpret_cast<std::remove_reference_t<decltype(ptr)>>(p);
    p += sz[k++];
  };
  take(b->keys); take(b->pair_box); take(b->freq); take(b->rank); take(b->box_mask);
  take(b->sort_key); take(b->word_a); take(b->word_b); take(b->tile_mask); take(b->order_a);
  take(b->order_b); take(b->pos); take(b->counts); take(b->lpt); take(b->inv_lpt);
  take(b->key_start);
  b->cub_tmp = p;
  b->cub_bytes = cub_bytes;
  p += sz[k++];
  take(b->status);

  auto fail = [&](cudaError_t err, const char *what) { return cuda_fail(err, what); };
  if ((e = cudaMemsetAsync(b->freq, 0, 4 * (size_t)K, s)) != cudaSuccess ||
      (e = cudaMemsetAsync(b->box_mask, 0, 8 * (size_t)n * W, s)) != cudaSuccess ||
      (e = cudaMemsetAsync(b->tile_mask, 0, 8 * (size_t)std::max(T, 1) * W, s)) !=
          cudaSuccess ||
      (e = cudaMemsetAsync(b->status, 0, sizeof(SchedStatus), s)) != cudaSuccess)
    return fail(e, "cudaMemsetAsync(schedule builder)");
  if (n > 0)
    sched_classify_kernel<<<grid1d((int64_t)n * 32, 256), 256, 0, s>>>(
        plan->d, b->tree, nnz, W, b->keys, b->pair_box, b->box_mask, b->freq, b->status);
  if (b->tree.nboxes > 0)
    sched_check_modes_kernel<<<grid1d(b->tree.nboxes, 128), 128, 0, s>>>(b->tree, plan->d.nq,
                                                                         b->status);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(e, "schedule classify launch");

  // keys by frequency, rarest first (ties: key order)
  std::vector<int32_t> freq(K), rank(K), by(K);
  SchedStatus hs{};
  if ((e = cudaMemcpyAsync(freq.data(), b->freq, 4 * (size_t)K, cudaMemcpyDeviceToHost, s)) !=
          cudaSuccess ||
      (e = cudaMemcpyAsync(&hs, b->status, sizeof(hs), cudaMemcpyDeviceToHost, s)) !=
          cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return fail(e, "schedule builder: key frequencies");
  if ((st = sched_status_error(hs)) != VL1_OK) return st;
  std::iota(by.begin(), by.end(), 0);
  std::stable_sort(by.begin(), by.end(), [&](int a, int c) { return freq[a] < freq[c]; });
  for (int r = 0; r < K; ++r) rank[by[r]] = r;
  if ((e = cudaMemcpyAsync(b->rank, rank.data(), 4 * (size_t)K, cudaMemcpyHostToDevice, s)) !=
      cudaSuccess)
    return fail(e, "schedule builder: key ranks");

  // boxes by sort key: stable LSD radix sort, least significant word first
  int32_t *order = b->order_a, *order_alt = b->order_b;
  if (n > 0) {
    sched_sort_key_kernel<<<grid1d(n, 128), 128, 0, s>>>(n, W, b->box_mask, b->rank,
                                                         b->sort_key);
    sched_iota_kernel<<<grid1d(n, 256), 256, 0, s>>>(n, order);
    for (int w = W - 1; w >= 0; --w) {
      sched_gather_word_kernel<<<grid1d(n, 256), 256, 0, s>>>(n, W, w, b->sort_key, order,
                                                              b->word_a);
      size_t tb = b->cub_bytes;
      if ((e = cub::DeviceRadixSort::SortPairs(b->cub_tmp, tb, b->word_a, b->word_b, order,
                                               order_alt, n, 0, 64, s)) != cudaSuccess)
        return fail(e, "schedule builder: radix sort");
      std::swap(order, order_alt);
    }
    b->order_a = order;
    b->order_b = order_alt;
    sched_inverse_kernel<<<grid1d(n, 256), 256, 0, s>>>(n, order, b->pos);
    sched_tile_mask_kernel<<<grid1d((int64_t)n * W, 256), 256, 0, s>>>(
        n, W, nrhs, b->box_mask, b->pos, b->tile_mask);
  }
  if (T > 0)
    sched_tile_count_kernel<<<grid1d(T, 256), 256, 0, s>>>(T, W, b->tile_mask, b->counts);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(e, "schedule tile launch");

  // tiles longest first (ties: tile order), their key starts
  std::vector<int32_t> counts(T), lpt(T), inv(T);
  if (T > 0 &&
      ((e = cudaMemcpyAsync(counts.data(), b->counts, 4 * (size_t)T, cudaMemcpyDeviceToHost,
                            s)) != cudaSuccess ||
       (e = cudaStreamSynchronize(s)) != cudaSuccess))
    return fail(e, "schedule builder: tile key counts");
  std::iota(lpt.begin(), lpt.end(), 0);
  std::stable_sort(lpt.begin(), lpt.end(), [&](int a, int c) { return counts[a] > counts[c]; });
  b->host_key_start.assign(T + 1, 0);
  for (int t = 0; t < T; ++t) {
    inv[lpt[t]] = t;
    b->host_key_start[t + 1] = b->host_key_start[t] + counts[lpt[t]];
  }
  b->n_entries = b->host_key_start[T];
  if (T > 0 &&
      ((e = cudaMemcpyAsync(b->lpt, lpt.data(), 4 * (size_t)T, cudaMemcpyHostToDevice, s)) !=
           cudaSuccess ||
       (e = cudaMemcpyAsync(b->inv_lpt, inv.data(), 4 * (size_t)T, cudaMemcpyHostToDevice,
                            s)) != cudaSuccess ||
       (e = cudaMemcpyAsync(b->key_start, b->host_key_start.data(), 4 * ((size_t)T + 1),
                            cudaMemcpyHostToDevice, s)) != cudaSuccess ||
       (e = cudaStreamSynchronize(s)) != cudaSuccess))
    return fail(e, "schedule builder: tile order");
  sizes->n_tiles = T;
  sizes->n_entries = b->n_entries;
  return VL1_OK;
}

}  // namespace

extern "C" int32_t vl1_schedule_build_key_start(const vl1_schedule_builder *b,
                                                int32_t *key_start_host) {
  if (!b || !key_start_host) {
    set_error("vl1_schedule_build_key_start: null argument");
    return VL1_E_ARG;
  }
  std::copy(b->host_key_start.begin(), b->host_key_start.end(), key_start_host);
  return VL1_OK;
}

extern "C" int32_t vl1_schedule_build_fill(vl1_schedule_builder *b, int32_t *tile_rows,
                                           int32_t *tile_key_start, int32_t *key_ids,
                                           int32_t *key_xrow, void *stream) {
  if (!b || (b->n_tiles > 0 && (!tile_rows || !tile_key_start)) ||
      (b->n_entries > 0 && (!key_ids || !key_xrow))) {
    set_error("vl1_schedule_build_fill: null argument");
    return VL1_E_ARG;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int T = b->n_tiles, W = b->words;
  cudaError_t e;
  if (T > 0) {
    sched_tile_rows_kernel<<<grid1d((int64_t)T * kTileRows, 256), 256, 0, s>>>(
        T, b->n_rows, b->nrhs, b->lpt, b->order_a, tile_rows);
    if ((e = cudaMemcpyAsync(tile_key_start, b->key_start, 4 * ((size_t)T + 1),
                             cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
      return cuda_fail(e, "vl1_schedule_build_fill: key starts");
    sched_key_ids_kernel<<<grid1d((int64_t)T * W, 128), 128, 0, s>>>(T, W, b->lpt, b->tile_mask,
                                                                    b->key_start, key_ids);
  }
  if (b->n_entries > 0) {
    if ((e = cudaMemsetAsync(key_xrow, 0xFF, 4 * (size_t)b->n_entries * kTileRows, s)) !=
        cudaSuccess)
      return cuda_fail(e, "vl1_schedule_build_fill: memset");
    sched_xrow_kernel<<<grid1d(b->nnz * b->nrhs, 256), 256, 0, s>>>(
        b->nnz, b->nrhs, W, b->keys, b->pair_box, b->tree.lists, b->pos, b->inv_lpt,
        b->key_start, b->tile_mask, key_xrow);
  }
  e = cudaGetLastError();
  return e == cudaSuccess ? VL1_OK : cuda_fail(e, "vl1_schedule_build_fill launch");
}

extern "C" int32_t vl1_schedule_builder_destroy(vl1_schedule_builder *b) {
  if (!b) return VL1_OK;
  cudaError_t e = b->buf ? cudaFreeAsync(b->buf, b->stream) : cudaSuccess;
  delete b;
  return e == cudaSuccess ? VL1_OK : cuda_fail(e, "cudaFreeAsync(schedule builder)");
}

// ---------------------------------------------------------------------------
// Work items of a schedule (host code; the cost model of the Python layer's
// MixedSchedule, run per new tree, so kept out of Python).

namespace {

// cost of one work item in units of one key's pipeline time: CTA start-up,
// pipeline drain and result write-back; the partial-sum write of a split
// part; the sum over the parts that the last part of a split tile reads back
// (fitted to measured launches of a 3D q = 4 tree over caps 12 .. 100000:
// within ~4 %)
constexpr double kItemOverheadKeys = 4.0;
constexpr double kSplitOverheadKeys = 1.5;
constexpr double kLastPartKeys = 2.0;
// candidate caps, as fractions of one SM's share of all keys
constexpr double kCapFractions[] = {1.5, 1.25, 1.0, 0.85, 0.75, 0.67, 0.6,
                                    0.5, 0.4, 0.33, 0.25, 0.2, 0.17};

struct SplitResult {
  std::vector<vl1_mixed_item> items;
  int n_splits = 0, n_slots = 0;
};

// tiles with more than `cap` keys split into nearly equal key ranges; items
// longest first (ties keep tile order)
SplitResult split_items(const int32_t *ks, int n_tiles, int cap) {
  SplitResult r;
  for (int t = 0; t < n_tiles; ++t) {
    const int k0 = ks[t], k1 = ks[t + 1], nk = k1 - k0;
    const int nparts = std::max(1, (nk + cap - 1) / cap);
    if (nparts == 1) {
      r.items.push_back(vl1_mixed_item{t, k0, k1, -1, 0, 1, -1, 0});
      continue;
    }
    for (int part = 0; part < nparts; ++part) {
      const int b0 = k0 + (int)(((int64_t)nk * part) / nparts);
      const int b1 = k0 + (int)(((int64_t)nk * (part + 1)) / nparts);
      r.items.push_back(vl1_mixed_item{t, b0, b1, r.n_splits, part, nparts, r.n_slots + part, 0});
    }
    ++r.n_splits;
    r.n_slots += nparts;
  }
  std::stable_sort(r.items.begin(), r.items.end(),
                   [](const vl1_mixed_item &a, const vl1_mixed_item &b) {
                     return (a.key_end - a.key_begin) > (b.key_end - b.key_begin);
                   });
  return r;
}

double item_cost(const vl1_mixed_item &it) {
  double c = (it.key_end - it.key_begin) + kItemOverheadKeys;
  if (it.split >= 0) c += kSplitOverheadKeys + (it.part == it.nparts - 1 ? kLastPartKeys : 0.0);
  return c;
}

// lower bound of the finish time: the longest item, and the mean load per slot
double makespan_bound(const std::vector<vl1_mixed_item> &items, int n_sm) {
  if (items.empty()) return 0.0;
  double mx = 0.0, sum = 0.0;
  for (const vl1_mixed_item &it : items) {
    const double c = item_cost(it);
    mx = std::max(mx, c);
    sum += c;
  }
  return std::max(mx, sum / n_sm);
}

// greedy list-scheduling finish time on n_sm one-CTA-per-SM slots, in order
double makespan(const std::vector<vl1_mixed_item> &items, int n_sm) {
  if ((int)items.size() <= n_sm) return items.empty() ? 0.0 : makespan_bound(items, n_sm);
  std::vector<double> heap(n_sm, 0.0);   // min-heap
  auto cmp = [](double a, double b) { return a > b; };
  for (const vl1_mixed_item &it : items) {
    std::pop_heap(heap.begin(), heap.end(), cmp);
    heap.back() += item_cost(it);
    std::push_heap(heap.begin(), heap.end(), cmp);
  }
  return *std::max_element(heap.begin(), heap.end());
}

}  // namespace

extern "C" int32_t vl1_mixed_work_items(const int32_t *key_start, int32_t n_tiles, int32_t cap,
                                        int32_t n_sm, vl1_mixed_item *items, int32_t capacity,
                                        int32_t *n_items, int32_t *n_splits,
                                        int32_t *n_slots) {
  if (!key_start || n_tiles < 0 || n_sm < 1 || !n_items || !n_splits || !n_slots) {
    set_error("vl1_mixed_work_items: null argument, n_tiles < 0 or n_sm < 1");
    return VL1_E_ARG;
  }
  for (int t = 0; t < n_tiles; ++t)
    if (key_start[t + 1] < key_start[t]) {
      set_error("vl1_mixed_work_items: key_start decreases at tile %d", t);
      return VL1_E_ARG;
    }
  SplitResult best;
  if (cap > 0) {
    best = split_items(key_start, n_tiles, cap);
  } else {
    const int64_t total = key_start[n_tiles];
    const int64_t share = std::max<int64_t>(1, (total + n_sm - 1) / n_sm);
    double best_t = 0.0;
    bool have = false;
    std::vector<int> seen;
    for (double f : kCapFractions) {
      const int c = std::max(4, (int)std::ceil((double)share * f));
      if (std::find(seen.begin(), seen.end(), c) != seen.end()) continue;
      seen.push_back(c);
      SplitResult cand = split_items(key_start, n_tiles, c);
      if (have && makespan_bound(cand.items, n_sm) > best_t) continue;
      const double t = makespan(cand.items, n_sm);
      if (!have || t < best_t) {
        best_t = t;
        best = std::move(cand);
        have = true;
      }
    }
  }
  *n_items = (int32_t)best.items.size();
  *n_splits = best.n_splits;
  *n_slots = best.n_slots;
  if (!items || capacity < (int32_t)best.items.size()) {
    set_error("vl1_mixed_work_items: %d items need room, %d given", (int)best.items.size(),
              capacity);
    return VL1_E_ARG;
  }
  std::copy(best.items.begin(), best.items.end(), items);
  return VL1_OK;
}
