// Box keys and an open-addressed device hash table of box keys, shared by
// the list-1 CSR builder and the tree builder.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace vl1 {

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  // MurmurHash3's 64-bit finaliser (public domain): spreads keys over the table
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return x;
}

// boxes of levels below `lev`: sum_{j<lev} 2^(dim j)
__host__ __device__ __forceinline__ long long level_offset(int dim, int lev) {
  long long o = 0;
  for (int j = 0; j < lev; ++j) o += 1ll << (dim * j);
  return o;
}

// key = offset(level) + linear coordinates (axis 0 most significant): keys
// sort by level, then lexicographically by coordinates
__device__ __forceinline__ long long box_key(int dim, int lev, const long long *c) {
  long long k = 0;
  for (int a = 0; a < dim; ++a) k = (k << lev) | c[a];
  return level_offset(dim, lev) + k;
}

// open addressing with linear probing; keys -1 = empty
struct KeyHash {
  long long *keys;
  int32_t *vals;
  uint64_t mask;   // capacity - 1 (a power of two)

  // false when the table is full
  __device__ __forceinline__ bool insert(long long key, int32_t val) const {
    uint64_t h = mix64((uint64_t)key) & mask;
    for (uint64_t probe = 0; probe <= mask; ++probe) {
      const long long prev = (long long)atomicCAS(reinterpret_cast<unsigned long long *>(keys + h),
                                                  (unsigned long long)-1ll,
                                                  (unsigned long long)key);
      if (prev == -1ll || prev == key) {
        vals[h] = val;
        return true;
      }
      h = (h + 1) & mask;
    }
    return false;
  }

  __device__ __forceinline__ int32_t find(long long key) const {
    uint64_t h = mix64((uint64_t)key) & mask;
    for (uint64_t probe = 0; probe <= mask; ++probe) {
      const long long k = keys[h];
      if (k == key) return vals[h];
      if (k == -1ll) return -1;
      h = (h + 1) & mask;
    }
    return -1;
  }
};

// a power-of-two capacity of at least twice n
inline uint64_t hash_capacity(int64_t n) {
  uint64_t c = 64;
  while (c < 2ull * (uint64_t)(n > 0 ? n : 1)) c <<= 1;
  return c;
}

}  // namespace vl1
