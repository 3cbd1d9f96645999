// Box trees on the device: 2:1 level restriction of a set of leaves and the
// assembly of the particle tree of tensor Gauss-Legendre nodes.
//
// Level restriction (volumential/tree_interactive_build.py:202-432): a leaf
// at level L forces every leaf at a level below L - 1 that contains one of
// its same-level neighbour positions (its own position plus {-1,0,1}^d,
// inside the root box) to split into its 2^d children; passes repeat until
// no leaf is forced.  One pass: the leaves go into a hash table (box key ->
// leaf index), one thread per leaf looks up the ancestors of its neighbour
// positions at every level below L - 1 and flags the leaves it finds; the
// host reads the flag count (one synchronisation per pass) and a compaction
// writes the unflagged leaves and the children of the flagged ones.
//
// Assembly (the layout of build_particle_tree_from_box_tree,
// tree_interactive_build.py:1274-1441): the boxes are the leaves and all
// their ancestors, numbered by box key (level by level, lexicographically
// by integer coordinates inside a level: the keys of every leaf's ancestors
// are sorted and made unique on the device), box centres
// root_vertex + (coords + 0.5) * root_extent / 2^level, leaves in box order
// with q^d particles each (the tensor Gauss-Legendre nodes of the leaf in
// meshgrid "ij" order) and their weights.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cub/device/device_select.cuh>

#include <algorithm>
#include <vector>

#include "vl1_hash.cuh"
#include "vl1_internal.cuh"

namespace vl1 {
namespace {

constexpr int kTB = 256;

int tb_grid(int64_t n) {
  int64_t g = (n + kTB - 1) / kTB;
  if (g > 152 * 32) g = 152 * 32;
  return (int)(g < 1 ? 1 : g);
}

__global__ void tb_fill_kernel(long long *keys, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    keys[i] = -1ll;
}

__global__ void tb_hash_leaves_kernel(int dim, int n, const uint8_t *levels,
                                      const int32_t *coords, KeyHash h, int32_t *status) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    long long c[3];
    for (int a = 0; a < dim; ++a) c[a] = coords[i * dim + a];
    if (!h.insert(box_key(dim, levels[i], c), (int32_t)i)) atomicExch(status, 1);
  }
}

// flag[j] = 1 for every leaf j at a level below L - 1 that contains a
// same-level neighbour position of a leaf at level L
__global__ void tb_mark_kernel(int dim, int n, const uint8_t *levels, const int32_t *coords,
                               KeyHash h, int32_t *flag, int32_t *n_flagged) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int lev = levels[i];
    if (lev < 2) continue;
    long long c[3];
    for (int a = 0; a < dim; ++a) c[a] = coords[i * dim + a];
    const long long side = 1ll << lev;
    const int n3 = dim == 3 ? 27 : 9;
    for (int di = 0; di < n3; ++di) {
      long long pos[3];
      bool valid = true;
      int rem = di;
      for (int a = dim - 1; a >= 0; --a) {
        pos[a] = c[a] + (rem % 3 - 1);
        rem /= 3;
        valid = valid && pos[a] >= 0 && pos[a] < side;
      }
      if (!valid) continue;
      for (int coarse = 0; coarse < lev - 1; ++coarse) {
        long long anc[3];
        for (int a = 0; a < dim; ++a) anc[a] = pos[a] >> (lev - coarse);
        const int j = h.find(box_key(dim, coarse, anc));
        if (j >= 0 && atomicExch(flag + j, 1) == 0) atomicAdd(n_flagged, 1);
      }
    }
  }
}

// unflagged leaves as they are, flagged ones as their 2^d children
__global__ void tb_split_kernel(int dim, int n, const uint8_t *levels, const int32_t *coords,
                                const int32_t *flag, uint8_t *out_levels, int32_t *out_coords,
                                int32_t *n_out, int capacity, int32_t *status) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int nk = flag[i] ? (1 << dim) : 1;
    const int o = atomicAdd(n_out, nk);
    if (o + nk > capacity) {
      atomicExch(status, 2);
      continue;
    }
    if (nk == 1) {
      out_levels[o] = levels[i];
      for (int a = 0; a < dim; ++a) out_coords[(int64_t)o * dim + a] = coords[i * dim + a];
      continue;
    }
    for (int k = 0; k < nk; ++k) {
      out_levels[o + k] = (uint8_t)(levels[i] + 1);
      for (int a = 0; a < dim; ++a)
        out_coords[(int64_t)(o + k) * dim + a] =
            2 * coords[i * dim + a] + ((k >> (dim - 1 - a)) & 1);
    }
  }
}

// the keys of every leaf and of all its ancestors
__global__ void tb_ancestor_keys_kernel(int dim, int n, const uint8_t *levels,
                                        const int32_t *coords, const int64_t *key_start,
                                        long long *keys) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int lev = levels[i];
    long long c[3];
    for (int a = 0; a < dim; ++a) c[a] = coords[i * dim + a];
    long long *out = keys + key_start[i];
    for (int l = lev; l >= 0; --l) {
      long long anc[3];
      for (int a = 0; a < dim; ++a) anc[a] = c[a] >> (lev - l);
      out[lev - l] = box_key(dim, l, anc);
    }
  }
}

__global__ void tb_key_starts_kernel(int n, const uint8_t *levels, int64_t *counts) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    counts[i] = levels[i] + 1;
}

struct BoxOut {
  int dim, q, nboxes, n_leaves, max_level;
  int64_t aligned;
  double root_extent;
  double root_vertex[3];
  const long long *box_keys;   // [nboxes] sorted
  KeyHash leaf_hash;           // leaf keys -> leaf index in the balanced set
  uint8_t *levels;
  int32_t *coords;             // [nboxes][dim]
  double *centers;             // [dim][aligned]
  uint8_t *is_leaf;
  int32_t *iota;               // [nboxes]: the box ids (selected by the leaf flags)
};

__device__ __forceinline__ void decode_key(int dim, long long key, int &lev, long long *c) {
  lev = 0;
  while (level_offset(dim, lev + 1) <= key) ++lev;
  long long lin = key - level_offset(dim, lev);
  for (int a = dim - 1; a >= 0; --a) {
    c[a] = lin & ((1ll << lev) - 1);
    lin >>= lev;
  }
}

__global__ void tb_boxes_kernel(BoxOut B) {
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < B.nboxes;
       b += (int64_t)gridDim.x * blockDim.x) {
    int lev;
    long long c[3];
    const long long key = B.box_keys[b];
    decode_key(B.dim, key, lev, c);
    B.levels[b] = (uint8_t)lev;
    // extent = root_extent / 2^lev; centre = vertex + (coord + 0.5) * extent
    // (the host builder's operations, in its order)
    // (separately rounded operations: no contraction into fused multiply-adds)
    const double ext = __ddiv_rn(B.root_extent, (double)(1ll << lev));
    for (int a = 0; a < B.dim; ++a) {
      B.coords[b * B.dim + a] = (int32_t)c[a];
      B.centers[a * B.aligned + b] =
          __dadd_rn(B.root_vertex[a], __dmul_rn(__dadd_rn((double)c[a], 0.5), ext));
    }
    B.is_leaf[b] = B.leaf_hash.find(key) >= 0 ? 1 : 0;
    B.iota[b] = (int32_t)b;
  }
}

struct Particles {
  int dim, q, nq, n_leaves;
  int64_t aligned;
  double root_extent;
  const uint8_t *levels;
  const double *centers;
  const int32_t *leaf_boxes;   // [n_leaves]
  const double *ref;           // [dim][nq]: reference nodes on [-1, 1]
  const double *wref;          // [nq]: products of the 1D weights
  int32_t *starts, *counts;    // [nboxes]
  double *targets;             // [dim][n_leaves * nq]
  double *weights;             // [n_leaves * nq]
};

__global__ void tb_particles_kernel(Particles P) {
  const int64_t n = (int64_t)P.n_leaves * P.nq;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx / P.nq;
    const int j = (int)(idx - i * P.nq);
    const int b = P.leaf_boxes[i];
    // centre + (0.5 * extent) * node, separately rounded (the host's order)
    const double ext = __ddiv_rn(P.root_extent, (double)(1ll << P.levels[b]));
    const double half = __dmul_rn(0.5, ext);
    const int64_t N = (int64_t)P.n_leaves * P.nq;
    for (int a = 0; a < P.dim; ++a)
      P.targets[a * N + idx] =
          __dadd_rn(P.centers[a * P.aligned + b], __dmul_rn(half, P.ref[a * P.nq + j]));
    double hw = half;
    for (int a = 1; a < P.dim; ++a) hw = __dmul_rn(hw, half);
    P.weights[idx] = __dmul_rn(hw, P.wref[j]);
    if (j == 0) {
      P.starts[b] = (int32_t)(i * P.nq);
      P.counts[b] = P.nq;
    }
  }
}

}  // namespace
}  // namespace vl1

using namespace vl1;

struct vl1_tree_builder {
  int dim = 0, q = 0, n_leaves = 0, nboxes = 0, max_level = 0;
  int64_t aligned = 0;
  double root_extent = 0.0;
  double root_vertex[3] = {0, 0, 0};
  std::vector<void *> bufs;
  uint8_t *leaf_levels = nullptr;
  int32_t *leaf_coords = nullptr;
  long long *box_keys = nullptr;
  KeyHash leaf_hash{};
  std::vector<int32_t> level_start;   // host [max_level + 2]
};

namespace {

template <class T>
int32_t tb_alloc(vl1_tree_builder *b, T **out, size_t bytes) {
  void *p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes ? bytes : 16);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(tree builder)");
  b->bufs.push_back(p);
  *out = static_cast<T *>(p);
  return VL1_OK;
}

void tb_free(vl1_tree_builder *b) {
  for (void *p : b->bufs) cudaFree(p);
  b->bufs.clear();
}

// 2:1 balance of the leaves in place (levels / coords hold `capacity`)
int32_t balance(int dim, int32_t *n_leaves, int capacity, uint8_t *levels, int32_t *coords,
                cudaStream_t s) {
  int n = *n_leaves;
  std::vector<void *> tmp;
  auto alloc = [&](void **p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
    if (e == cudaSuccess) tmp.push_back(*p);
    return e;
  };
  auto release = [&]() {
    cudaStreamSynchronize(s);
    for (void *p : tmp) cudaFree(p);
  };
  uint8_t *lv2 = nullptr;
  int32_t *co2 = nullptr, *flag = nullptr, *ctr = nullptr;
  long long *hk = nullptr;
  int32_t *hv = nullptr;
  const uint64_t cap = hash_capacity(capacity);
  cudaError_t e;
  if ((e = alloc((void **)&lv2, (size_t)capacity)) != cudaSuccess ||
      (e = alloc((void **)&co2, 4 * (size_t)capacity * dim)) != cudaSuccess ||
      (e = alloc((void **)&flag, 4 * (size_t)capacity)) != cudaSuccess ||
      (e = alloc((void **)&ctr, 16)) != cudaSuccess ||
      (e = alloc((void **)&hk, 8 * cap)) != cudaSuccess ||
      (e = alloc((void **)&hv, 4 * cap)) != cudaSuccess) {
    release();
    return cuda_fail(e, "cudaMalloc(tree balance)");
  }
  KeyHash h{hk, hv, cap - 1};
  for (int pass = 0; pass < 64; ++pass) {
    int32_t host[4] = {0, 0, 0, 0};
    tb_fill_kernel<<<tb_grid((int64_t)cap), kTB, 0, s>>>(hk, (int64_t)cap);
    cudaMemsetAsync(flag, 0, 4 * (size_t)n, s);
    cudaMemsetAsync(ctr, 0, 16, s);
    tb_hash_leaves_kernel<<<tb_grid(n), kTB, 0, s>>>(dim, n, levels, coords, h, ctr + 2);
    tb_mark_kernel<<<tb_grid(n), kTB, 0, s>>>(dim, n, levels, coords, h, flag, ctr);
    if ((e = cudaMemcpyAsync(host, ctr, 16, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess) {
      release();
      return cuda_fail(e, "tree balance pass");
    }
    if (host[2]) {
      release();
      set_error("tree balance: hash table full");
      return VL1_E_NOMEM;
    }
    if (host[0] == 0) {
      release();
      *n_leaves = n;
      return VL1_OK;
    }
    const int64_t need = (int64_t)n + (int64_t)host[0] * ((1 << dim) - 1);
    if (need > capacity) {
      release();
      set_error("tree balance: %lld leaves need room, the capacity is %d", (long long)need,
                capacity);
      return VL1_E_ARG;
    }
    tb_split_kernel<<<tb_grid(n), kTB, 0, s>>>(dim, n, levels, coords, flag, lv2, co2, ctr + 1,
                                                capacity, ctr + 3);
    n = (int)need;
    cudaMemcpyAsync(levels, lv2, (size_t)n, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(coords, co2, 4 * (size_t)n * dim, cudaMemcpyDeviceToDevice, s);
    if ((e = cudaGetLastError()) != cudaSuccess) {
      release();
      return cuda_fail(e, "tree balance launch");
    }
  }
  release();
  set_error("tree balance did not converge in 64 passes");
  return VL1_E_ARG;
}

}  // namespace

extern "C" int32_t vl1_tree_balance(int32_t dim, int32_t *n_leaves, int32_t capacity,
                                    uint8_t *levels, int32_t *coords, void *stream) {
  if ((dim != 2 && dim != 3) || !n_leaves || *n_leaves < 1 || capacity < *n_leaves ||
      !levels || !coords) {
    set_error("vl1_tree_balance: dim not 2 or 3, no leaves, capacity below the leaf count "
              "or null arrays");
    return VL1_E_ARG;
  }
  return balance(dim, n_leaves, capacity, levels, coords, static_cast<cudaStream_t>(stream));
}

extern "C" int32_t vl1_tree_build_begin(int32_t dim, int32_t q, int32_t n_leaves,
                                        const uint8_t *leaf_levels, const int32_t *leaf_coords,
                                        double root_extent, const double *root_vertex,
                                        vl1_tree_builder **out, int32_t *sizes3,
                                        void *stream) {
  if ((dim != 2 && dim != 3) || q < 1 || n_leaves < 1 || !leaf_levels || !leaf_coords ||
      !root_vertex || !out || !sizes3 || !(root_extent > 0)) {
    set_error("vl1_tree_build_begin: invalid argument");
    return VL1_E_ARG;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  vl1_tree_builder *b = new vl1_tree_builder();
  b->dim = dim;
  b->q = q;
  b->n_leaves = n_leaves;
  b->root_extent = root_extent;
  for (int a = 0; a < dim; ++a) b->root_vertex[a] = root_vertex[a];
  auto fail = [&](int32_t st) {
    cudaStreamSynchronize(s);
    tb_free(b);
    delete b;
    return st;
  };
  int32_t st;
  cudaError_t e;
  // leaf keys with all ancestors: per leaf (level + 1) keys
  int64_t *kcount = nullptr, *kstart = nullptr;
  long long *all = nullptr, *sorted = nullptr;
  int32_t *n_unique = nullptr;
  if ((st = tb_alloc(b, &kcount, 8 * (size_t)n_leaves))) return fail(st);
  if ((st = tb_alloc(b, &kstart, 8 * ((size_t)n_leaves + 1)))) return fail(st);
  tb_key_starts_kernel<<<tb_grid(n_leaves), kTB, 0, s>>>(n_leaves, leaf_levels, kcount);
  size_t scan_bytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, kcount, kstart, n_leaves, s);
  void *scan_tmp = nullptr;
  if ((st = tb_alloc(b, &scan_tmp, scan_bytes))) return fail(st);
  cub::DeviceScan::ExclusiveSum(scan_tmp, scan_bytes, kcount, kstart, n_leaves, s);
  int64_t last[2] = {0, 0};
  if ((e = cudaMemcpyAsync(&last[0], kstart + n_leaves - 1, 8, cudaMemcpyDeviceToHost, s)) !=
          cudaSuccess ||
      (e = cudaMemcpyAsync(&last[1], kcount + n_leaves - 1, 8, cudaMemcpyDeviceToHost, s)) !=
          cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return fail(cuda_fail(e, "tree build: key count"));
  const int64_t n_keys = last[0] + last[1];
  if ((st = tb_alloc(b, &all, 8 * (size_t)n_keys))) return fail(st);
  if ((st = tb_alloc(b, &sorted, 8 * (size_t)n_keys))) return fail(st);
  if ((st = tb_alloc(b, &n_unique, 16))) return fail(st);
  tb_ancestor_keys_kernel<<<tb_grid(n_leaves), kTB, 0, s>>>(dim, n_leaves, leaf_levels,
                                                           leaf_coords, kstart, all);
  size_t sort_bytes = 0, uniq_bytes = 0;
  cub::DeviceRadixSort::SortKeys(nullptr, sort_bytes, all, sorted, (int)n_keys, 0, 64, s);
  cub::DeviceSelect::Unique(nullptr, uniq_bytes, sorted, all, n_unique, (int)n_keys, s);
  void *tmp = nullptr;
  if ((st = tb_alloc(b, &tmp, std::max(sort_bytes, uniq_bytes)))) return fail(st);
  cub::DeviceRadixSort::SortKeys(tmp, sort_bytes, all, sorted, (int)n_keys, 0, 64, s);
  cub::DeviceSelect::Unique(tmp, uniq_bytes, sorted, all, n_unique, (int)n_keys, s);
  int32_t nb = 0;
  if ((e = cudaMemcpyAsync(&nb, n_unique, 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return fail(cuda_fail(e, "tree build: box count"));
  b->nboxes = nb;
  b->box_keys = all;   // the first nb keys, sorted and distinct
  // levels from the key ranges (level starts)
  std::vector<long long> keys_host((size_t)nb);
  if ((e = cudaMemcpyAsync(keys_host.data(), all, 8 * (size_t)nb, cudaMemcpyDeviceToHost, s)) !=
          cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return fail(cuda_fail(e, "tree build: box keys"));
  int lev = 0;
  while (level_offset(dim, lev + 1) <= keys_host[nb - 1]) ++lev;
  b->max_level = lev;
  b->level_start.assign(lev + 2, 0);
  for (int l = 0; l <= lev + 1; ++l)
    b->level_start[l] = (int32_t)(std::lower_bound(keys_host.begin(), keys_host.end(),
                                                   level_offset(dim, l)) - keys_host.begin());
  // leaf hash (leaf keys)
  const uint64_t cap = hash_capacity(n_leaves);
  long long *hk = nullptr;
  int32_t *hv = nullptr, *hstat = nullptr;
  if ((st = tb_alloc(b, &hk, 8 * cap)) || (st = tb_alloc(b, &hv, 4 * cap)) ||
      (st = tb_alloc(b, &hstat, 4)))
    return fail(st);
  tb_fill_kernel<<<tb_grid((int64_t)cap), kTB, 0, s>>>(hk, (int64_t)cap);
  cudaMemsetAsync(hstat, 0, 4, s);
  b->leaf_hash = KeyHash{hk, hv, cap - 1};
  tb_hash_leaves_kernel<<<tb_grid(n_leaves), kTB, 0, s>>>(dim, n_leaves, leaf_levels,
                                                          leaf_coords, b->leaf_hash, hstat);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(cuda_fail(e, "tree build launch"));
  b->aligned = ((int64_t)nb + 31) / 32 * 32;
  sizes3[0] = nb;
  sizes3[1] = (int32_t)b->aligned;
  sizes3[2] = lev;
  *out = b;
  return VL1_OK;
}

extern "C" int32_t vl1_tree_build_level_starts(const vl1_tree_builder *b, int32_t *out) {
  if (!b || !out) {
    set_error("vl1_tree_build_level_starts: null argument");
    return VL1_E_ARG;
  }
  std::copy(b->level_start.begin(), b->level_start.end(), out);
  return VL1_OK;
}

extern "C" int32_t vl1_tree_build_fill(vl1_tree_builder *b, const double *ref_nodes,
                                       const double *ref_weights, uint8_t *box_levels,
                                       int32_t *box_coords, double *box_centers,
                                       uint8_t *box_is_leaf, int32_t *box_starts,
                                       int32_t *box_counts, int32_t *leaf_boxes,
                                       double *targets, double *weights, void *stream) {
  if (!b || !ref_nodes || !ref_weights || !box_levels || !box_coords || !box_centers ||
      !box_is_leaf || !box_starts || !box_counts || !leaf_boxes || !targets || !weights) {
    set_error("vl1_tree_build_fill: null argument");
    return VL1_E_ARG;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nb = b->nboxes;
  int32_t *iota = nullptr, *n_sel = nullptr;
  int32_t st;
  if ((st = tb_alloc(b, &iota, 4 * (size_t)nb)) || (st = tb_alloc(b, &n_sel, 16))) return st;
  cudaMemsetAsync(box_centers, 0, 8 * (size_t)b->dim * b->aligned, s);
  cudaMemsetAsync(box_starts, 0, 4 * (size_t)nb, s);
  cudaMemsetAsync(box_counts, 0, 4 * (size_t)nb, s);
  BoxOut B;
  B.dim = b->dim;
  B.q = b->q;
  B.nboxes = nb;
  B.n_leaves = b->n_leaves;
  B.max_level = b->max_level;
  B.aligned = b->aligned;
  B.root_extent = b->root_extent;
  for (int a = 0; a < 3; ++a) B.root_vertex[a] = b->root_vertex[a];
  B.box_keys = b->box_keys;
  B.leaf_hash = b->leaf_hash;
  B.levels = box_levels;
  B.coords = box_coords;
  B.centers = box_centers;
  B.is_leaf = box_is_leaf;
  B.iota = iota;
  tb_boxes_kernel<<<tb_grid(nb), kTB, 0, s>>>(B);
  // leaf boxes in box order: the indices of the leaf flags
  size_t sel_bytes = 0;
  cub::DeviceSelect::Flagged(nullptr, sel_bytes, iota, box_is_leaf, leaf_boxes, n_sel, nb, s);
  void *tmp = nullptr;
  if ((st = tb_alloc(b, &tmp, sel_bytes))) return st;
  cub::DeviceSelect::Flagged(tmp, sel_bytes, iota, box_is_leaf, leaf_boxes, n_sel, nb, s);
  int nq = 1;
  for (int a = 0; a < b->dim; ++a) nq *= b->q;
  double *ref = nullptr, *wref = nullptr;
  if ((st = tb_alloc(b, &ref, 8 * (size_t)b->dim * nq)) ||
      (st = tb_alloc(b, &wref, 8 * (size_t)nq)))
    return st;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(ref, ref_nodes, 8 * (size_t)b->dim * nq, cudaMemcpyHostToDevice,
                           s)) != cudaSuccess ||
      (e = cudaMemcpyAsync(wref, ref_weights, 8 * (size_t)nq, cudaMemcpyHostToDevice, s)) !=
          cudaSuccess)
    return cuda_fail(e, "tree build: reference nodes");
  Particles P;
  P.dim = b->dim;
  P.q = b->q;
  P.nq = nq;
  P.n_leaves = b->n_leaves;
  P.aligned = b->aligned;
  P.root_extent = b->root_extent;
  P.levels = box_levels;
  P.centers = box_centers;
  P.leaf_boxes = leaf_boxes;
  P.ref = ref;
  P.wref = wref;
  P.starts = box_starts;
  P.counts = box_counts;
  P.targets = targets;
  P.weights = weights;
  tb_particles_kernel<<<tb_grid((int64_t)b->n_leaves * nq), kTB, 0, s>>>(P);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "tree build fill launch");
  // the host reference arrays above are read by the copies: finish them
  e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? VL1_OK : cuda_fail(e, "tree build fill");
}

extern "C" int32_t vl1_tree_builder_destroy(vl1_tree_builder *b) {
  if (!b) return VL1_OK;
  tb_free(b);
  delete b;
  return VL1_OK;
}
