// Blackwell (sm_100 family) tensor-core, TMEM, mbarrier and bulk-copy helpers
// written as inline PTX.  Every wait on an mbarrier is bounded.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace vl1 {
namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---------------------------------------------------------------- mbarrier
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

// Test the phase parity; the thread may sleep (up to `hint_ns`) until the
// phase completes instead of returning at once; a sleeping warp takes no
// issue slots from the warps doing work.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t *bar, uint32_t phase,
                                                    uint32_t hint_ns) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(phase), "r"(hint_ns)
      : "memory");
  return ok != 0;
}

// ------------------------------------------------------- bulk copy (1D TMA)
// global -> shared, completion counted on `bar` (bytes, 16-byte multiples,
// both addresses 16-byte aligned)
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// ---------------------------------------------------- cp.async (16 bytes)
// 16 bytes, of which the first `src_bytes` (0 or 16) are read and the rest
// zero-filled; with src_bytes == 0 nothing is read from `src`
__device__ __forceinline__ void cp_async16_zfill(void *dst, const void *src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_addr(dst)), "l"(src),
               "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
// wait until at most N of this thread's committed cp.async groups are pending
template <int N>
__device__ __forceinline__ void cp_async_wait_group() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

// arrive on `bar` once every cp.async this thread issued before has landed;
// the arrival counts as one of the barrier's expected arrivals (.noinc)
__device__ __forceinline__ void cp_async_mbar_arrive_noinc(uint64_t *bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

// make generic-proxy writes to shared memory visible to the async proxy
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---------------------------------------------------------------- TMEM
__device__ __forceinline__ void tmem_alloc(uint32_t *dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
               ::"r"(smem_addr(dst_smem)), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// 32 lanes x 16 consecutive 32-bit columns -> 16 registers per thread
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
        "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
        "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// ------------------------------------------------------------------ MMA
// Shared-memory matrix descriptor, K-major, swizzled rows of `row_bytes`
// (32, 64 or 128 bytes = 16, 32 or 64 16-bit values along K).  Eight rows form one
// swizzle atom of 8 * row_bytes bytes (aligned to that size); the 16-byte
// chunk c of row r sits at chunk c ^ (bits 7.. of the row's offset), as the
// hardware applies it to absolute shared-memory addresses.
//   sbo: byte distance between atoms adjacent along M/N (8 * row_bytes)
__device__ __forceinline__ uint64_t smem_desc_kmajor_swizzled(uint32_t saddr, uint32_t row_bytes) {
  const uint64_t layout = row_bytes == 128 ? 2 : (row_bytes == 64 ? 4 : 6);
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;                                   // lbo (unused): 16 bytes
  d |= (uint64_t)(((8 * row_bytes) >> 4) & 0x3FFF) << 32;   // sbo
  d |= (uint64_t)1 << 46;
  d |= layout << 61;
  return d;
}

// Byte offset of element (row, k) in a K-major swizzled operand with `kc`
// 16-bit values per row (row bytes 2*kc in {32, 64, 128}), relative to an atom-aligned
// base.
__host__ __device__ __forceinline__ uint32_t kmajor_swizzled_offset(uint32_t row, uint32_t k,
                                                                    uint32_t kc) {
  const uint32_t row_bytes = 2u * kc;
  const uint32_t mask = row_bytes / 16u - 1u;
  const uint32_t a = (row & 7u) * row_bytes + (k >> 3) * 16u + (k & 7u) * 2u;
  const uint32_t chunk = ((a >> 4) & mask) ^ ((a >> 7) & mask);
  return (row >> 3) * 8u * row_bytes + (a & ~(mask << 4)) + (chunk << 4);
}

// Instruction descriptor of kind::f16: F16 x F16 -> FP32, both K-major.
__host__ __device__ constexpr uint32_t idesc_f16_f32(int m, int n) {
  return (1u << 4)                          // D format: F32 (A, B format 0: F16)
         | ((uint32_t)(n >> 3) << 17)       // N / 8
         | ((uint32_t)(m >> 4) << 24);      // M / 16
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread (kind::f16 with the
// F16 x F16 instruction descriptor above)
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(d_tmem), "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// arrive on `bar` when every prior tcgen05.mma of this thread has completed
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
      ::"r"(smem_addr(bar))
      : "memory");
}

}  // namespace tc
}  // namespace vl1
