// List-1 CSR on the device: for every leaf (target box), the leaves that
// touch it at its own level, one level coarser or one level finer (the
// list-1 interaction list of a 2:1-balanced tree; the reference takes it from
// boxtree's FMMTraversalBuilder, used at volumential/volume_fmm.py:984-989).
//
// Boxes are named by key = offset(level) + linear(coordinates at that level)
// (offset(l) = sum_{j<l} 2^(d j), coordinates axis 0 most significant).
// Leaves go into an open-addressed hash table (key -> box id); one thread per
// target leaf enumerates the candidate positions with the validity rules of
// the host builder:
//   same level: coords + delta, delta in {-1,0,1}^d (the leaf itself included);
//   one coarser: (coords + delta) >> 1 for in-range coords + delta, unless
//                that is the leaf's parent (each such cell once);
//   one finer:   2 coords + delta, delta in {-1,0,1,2}^d minus {0,1}^d;
// and looks them up; the hits are distinct boxes, so the count pass only
// counts and the fill pass sorts its row.  Count, exclusive scan (three
// launches over tiles of 4096 counts) and fill are separate launches; the
// row order is ascending box id.

#include <cuda_runtime.h>

#include <cstdint>

#include "vl1_hash.cuh"
#include "vl1_internal.cuh"

namespace vl1 {
namespace {

constexpr int kMaxCand = 27 + 8 + 56;   // 3D: same + coarser + finer
constexpr int kTreeThreads = 256;
constexpr int kScanThreads = 1024;
constexpr int kScanTile = 4 * kScanThreads;   // counts per scan block

struct CsrArgs {
  int dim, nboxes, n_leaves, max_level;
  const uint8_t *levels;
  const int32_t *coords;      // [nboxes][dim]
  const int32_t *leaf_boxes;  // [n_leaves]
  long long *hkeys;           // [cap], -1 empty
  int32_t *hvals;             // [cap]
  uint64_t cap_mask;
  int32_t *counts;            // [n_leaves + 1]
  long long *tile_sums;       // [n_leaves / kScanTile + 1]
  int32_t *starts;            // [n_leaves + 1]
  int32_t *lists;
  int32_t *status;            // [1]: 0 ok, 1 table full, 2 bad input
};

__global__ void hash_insert_kernel(const CsrArgs A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.n_leaves) return;
  const int b = A.leaf_boxes[i];
  if (b < 0 || b >= A.nboxes) {
    atomicExch(A.status, 2);
    return;
  }
  const int lev = A.levels[b];
  long long c[3];
  for (int a = 0; a < A.dim; ++a) c[a] = A.coords[(int64_t)b * A.dim + a];
  const long long key = box_key(A.dim, lev, c);
  uint64_t h = mix64((uint64_t)key) & A.cap_mask;
  for (uint64_t probe = 0; probe <= A.cap_mask; ++probe) {
    const long long prev =
        atomicCAS(reinterpret_cast<unsigned long long *>(A.hkeys + h), (unsigned long long)-1ll,
                  (unsigned long long)key);
    if (prev == -1ll || prev == key) {
      A.hvals[h] = b;
      return;
    }
    h = (h + 1) & A.cap_mask;
  }
  atomicExch(A.status, 1);
}

__device__ __forceinline__ int hash_find(const CsrArgs &A, long long key) {
  uint64_t h = mix64((uint64_t)key) & A.cap_mask;
  for (uint64_t probe = 0; probe <= A.cap_mask; ++probe) {
    const long long k = A.hkeys[h];
    if (k == key) return A.hvals[h];
    if (k == -1ll) return -1;
    h = (h + 1) & A.cap_mask;
  }
  return -1;
}

// The list-1 boxes of target leaf i: the leaves at its own level at
// coords + delta, delta in {-1,0,1}^d (itself included); the leaves one
// level coarser that contain such a position, except its parent; the leaves
// one level finer at 2 coords + delta, delta in {-1..2}^d outside {0,1}^d.
// Every hit is a distinct box: the same-level and finer positions are
// distinct, and the coarser cells are enumerated once each (per axis the
// distinct values of (coords + delta) >> 1 over the in-range deltas, at
// most two).  EMIT(id) is called per hit; returns the number of hits.
template <class Emit>
__device__ __forceinline__ int leaf_hits(const CsrArgs &A, int i, Emit emit) {
  const int dim = A.dim;
  const int b = A.leaf_boxes[i];
  if (b < 0 || b >= A.nboxes) return 0;   // reported by the insert kernel
  const int tl = A.levels[b];
  long long tc[3];
  for (int a = 0; a < dim; ++a) tc[a] = A.coords[(int64_t)b * dim + a];
  const long long side = 1ll << tl;
  int n = 0;
  // same level
  const int n3 = dim == 3 ? 27 : 9;
  for (int di = 0; di < n3; ++di) {
    long long pos[3];
    bool valid = true;
    int rem = di;
    for (int a = dim - 1; a >= 0; --a) {
      const int d = rem % 3 - 1;
      rem /= 3;
      pos[a] = tc[a] + d;
      valid = valid && pos[a] >= 0 && pos[a] < side;
    }
    if (!valid) continue;
    const int id = hash_find(A, box_key(dim, tl, pos));
    if (id >= 0) {
      emit(n, id);
      ++n;
    }
  }
  // one coarser: per axis the distinct parents of the in-range positions
  if (tl >= 1) {
    long long cv[3][2];
    int nv[3];
    for (int a = 0; a < dim; ++a) {
      nv[a] = 0;
      for (int d = -1; d <= 1; ++d) {
        const long long p = tc[a] + d;
        if (p < 0 || p >= side) continue;
        const long long c = p >> 1;
        if (nv[a] == 0 || cv[a][nv[a] - 1] != c) cv[a][nv[a]++] = c;   // ascending
      }
    }
    const int tot = dim == 3 ? nv[0] * nv[1] * nv[2] : nv[0] * nv[1];
    for (int ci = 0; ci < tot; ++ci) {
      long long cp[3];
      bool parent = true;
      int rem = ci;
      for (int a = dim - 1; a >= 0; --a) {
        cp[a] = cv[a][rem % nv[a]];
        rem /= nv[a];
        parent = parent && cp[a] == (tc[a] >> 1);
      }
      if (parent) continue;   // the leaf's own ancestor
      const int id = hash_find(A, box_key(dim, tl - 1, cp));
      if (id >= 0) {
        emit(n, id);
        ++n;
      }
    }
  }
  // one finer: 2 coords + delta, delta in {-1..2}^d outside {0,1}^d
  if (tl + 1 <= A.max_level) {
    const int n4 = dim == 3 ? 64 : 16;
    for (int di = 0; di < n4; ++di) {
      long long pos[3];
      bool valid = true, inner = true;
      int rem = di;
      for (int a = dim - 1; a >= 0; --a) {
        const int d = rem % 4 - 1;
        rem /= 4;
        pos[a] = 2 * tc[a] + d;
        inner = inner && (d == 0 || d == 1);
        valid = valid && pos[a] >= 0 && pos[a] < 2 * side;
      }
      if (inner || !valid) continue;
      const int id = hash_find(A, box_key(dim, tl + 1, pos));
      if (id >= 0) {
        emit(n, id);
        ++n;
      }
    }
  }
  return n;
}

// candidates of target leaf i, sorted ascending; returns their number
__device__ int leaf_candidates(const CsrArgs &A, int i, int *out) {
  const int n = leaf_hits(A, i, [&](int k, int id) { out[k] = id; });
  for (int x = 1; x < n; ++x) {   // insertion sort
    const int v = out[x];
    int y = x - 1;
    while (y >= 0 && out[y] > v) {
      out[y + 1] = out[y];
      --y;
    }
    out[y + 1] = v;
  }
  return n;
}

__global__ void csr_count_kernel(const CsrArgs A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.n_leaves) return;
  A.counts[i] = leaf_hits(A, i, [](int, int) {});   // distinct hits: no sort needed
}

// exclusive scan of counts[0..n) into starts[0..n] in three launches: the sum
// of every tile of kScanTile counts, an exclusive scan of the tile sums (one
// CTA), then each tile's scan from its offset.

// inclusive block scan of one value per thread (warp shuffles, then the warp
// totals in shared memory); `total` receives the block's sum
__device__ __forceinline__ long long block_inclusive_scan(long long v, long long *s_warp,
                                                         long long &total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  if (lane == 31) s_warp[wid] = v;
  __syncthreads();
  if (wid == 0) {
    long long w = lane < (int)(blockDim.x >> 5) ? s_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long u = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += u;
    }
    s_warp[lane] = w;   // inclusive warp-total prefix
  }
  __syncthreads();
  total = s_warp[(blockDim.x >> 5) - 1];
  const long long add = wid > 0 ? s_warp[wid - 1] : 0;
  __syncthreads();
  return v + add;
}

__global__ void __launch_bounds__(kScanThreads) csr_tile_sum_kernel(const CsrArgs A) {
  __shared__ long long s_warp[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + 4 * threadIdx.x;
  long long v = 0;
#pragma unroll
  for (int j = 0; j < 4; ++j)
    if (base + j < A.n_leaves) v += A.counts[base + j];
  long long total;
  block_inclusive_scan(v, s_warp, total);
  if (threadIdx.x == 0) A.tile_sums[blockIdx.x] = total;
}

// one CTA: exclusive scan of the n_tiles tile sums in place; starts[n] = total
__global__ void __launch_bounds__(kScanThreads) csr_tile_scan_kernel(const CsrArgs A,
                                                                     int n_tiles) {
  __shared__ long long s_warp[32];
  long long carry = 0;
  for (int t0 = 0; t0 < n_tiles; t0 += kScanThreads) {
    const int t = t0 + threadIdx.x;
    const long long v = t < n_tiles ? A.tile_sums[t] : 0;
    long long total;
    const long long inc = block_inclusive_scan(v, s_warp, total);
    if (t < n_tiles) A.tile_sums[t] = carry + inc - v;
    carry += total;
  }
  if (threadIdx.x == 0) {
    if (carry > 0x7fffffffll) atomicExch(A.status, 2);
    A.starts[A.n_leaves] = (int32_t)carry;
  }
}

__global__ void __launch_bounds__(kScanThreads) csr_tile_down_kernel(const CsrArgs A) {
  __shared__ long long s_warp[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + 4 * threadIdx.x;
  int c[4];
  long long v = 0;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    c[j] = base + j < A.n_leaves ? A.counts[base + j] : 0;
    v += c[j];
  }
  long long total;
  long long run = block_inclusive_scan(v, s_warp, total) - v + A.tile_sums[blockIdx.x];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    if (base + j < A.n_leaves) A.starts[base + j] = (int32_t)run;
    run += c[j];
  }
}

__global__ void csr_fill_kernel(const CsrArgs A, int64_t capacity) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.n_leaves) return;
  int cand[kMaxCand];
  const int m = leaf_candidates(A, i, cand);
  const int64_t s = A.starts[i];
  if (s + m > capacity) {
    atomicExch(A.status, 1);
    return;
  }
  for (int x = 0; x < m; ++x) A.lists[s + x] = cand[x];
}

}  // namespace
}  // namespace vl1

using namespace vl1;

namespace {
uint64_t table_capacity(int32_t n_leaves) {
  uint64_t cap = 64;
  while (cap < 2ull * (uint64_t)n_leaves) cap <<= 1;
  return cap;
}
}  // namespace

extern "C" int64_t vl1_list1_csr_workspace_bytes(int32_t n_leaves) {
  if (n_leaves < 0) return -1;
  const uint64_t cap = table_capacity(n_leaves);
  const uint64_t n_tiles = ((uint64_t)n_leaves + kScanTile - 1) / kScanTile + 1;
  return (int64_t)(cap * 8 + cap * 4 + ((uint64_t)n_leaves + 1) * 4 + 256 + n_tiles * 8);
}

extern "C" int32_t vl1_list1_csr(const vl1_csr_desc *desc, int64_t *nnz, void *stream) {
  if (!desc || !nnz) {
    set_error("vl1_list1_csr: null argument");
    return VL1_E_ARG;
  }
  const vl1_csr_desc &D = *desc;
  if ((D.dim != 2 && D.dim != 3) || D.nboxes < 1 || D.n_leaves < 1 || D.max_level < 0 ||
      D.max_level > (D.dim == 3 ? 20 : 30) || !D.box_levels || !D.box_coords ||
      !D.leaf_boxes || !D.starts || !D.lists || !D.workspace ||
      D.workspace_bytes < vl1_list1_csr_workspace_bytes(D.n_leaves)) {
    set_error("vl1_list1_csr: dim %d, %d boxes, %d leaves, max level %d or workspace "
              "out of range", D.dim, D.nboxes, D.n_leaves, D.max_level);
    return VL1_E_ARG;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const uint64_t cap = table_capacity(D.n_leaves);
  uint8_t *w = static_cast<uint8_t *>(D.workspace);
  CsrArgs A;
  A.dim = D.dim;
  A.nboxes = D.nboxes;
  A.n_leaves = D.n_leaves;
  A.max_level = D.max_level;
  A.levels = D.box_levels;
  A.coords = D.box_coords;
  A.leaf_boxes = D.leaf_boxes;
  A.hkeys = reinterpret_cast<long long *>(w);
  A.hvals = reinterpret_cast<int32_t *>(w + cap * 8);
  A.counts = reinterpret_cast<int32_t *>(w + cap * 12);
  A.status = reinterpret_cast<int32_t *>(w + cap * 12 + ((uint64_t)D.n_leaves + 1) * 4);
  // 8-byte aligned: the status word's 256-byte slot, then the tile sums
  A.tile_sums = reinterpret_cast<long long *>(
      w + ((cap * 12 + ((uint64_t)D.n_leaves + 1) * 4 + 256 + 7) & ~(uint64_t)7));
  A.cap_mask = cap - 1;
  A.starts = D.starts;
  A.lists = D.lists;
  cudaError_t e = cudaMemsetAsync(A.hkeys, 0xFF, cap * 8, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(A.status, 0, 4, s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(list-1 csr)");
  const int grid = (D.n_leaves + kTreeThreads - 1) / kTreeThreads;
  hash_insert_kernel<<<grid, kTreeThreads, 0, s>>>(A);
  csr_count_kernel<<<grid, kTreeThreads, 0, s>>>(A);
  const int n_tiles = (int)(((int64_t)D.n_leaves + kScanTile - 1) / kScanTile);
  csr_tile_sum_kernel<<<n_tiles, kScanThreads, 0, s>>>(A);
  csr_tile_scan_kernel<<<1, kScanThreads, 0, s>>>(A, n_tiles);
  csr_tile_down_kernel<<<n_tiles, kScanThreads, 0, s>>>(A);
  csr_fill_kernel<<<grid, kTreeThreads, 0, s>>>(A, D.lists_capacity);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "list-1 csr launches");
  int32_t host[2];
  e = cudaMemcpyAsync(&host[0], A.status, 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&host[1], D.starts + D.n_leaves, 4,
                                            cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "list-1 csr read-back");
  if (host[0] == 1) {
    set_error("vl1_list1_csr: list capacity %lld too small", (long long)D.lists_capacity);
    return VL1_E_ARG;
  }
  if (host[0] == 2) {
    set_error("vl1_list1_csr: invalid leaf box id or more than 2^31 list entries");
    return VL1_E_ARG;
  }
  *nnz = host[1];
  return VL1_OK;
}
