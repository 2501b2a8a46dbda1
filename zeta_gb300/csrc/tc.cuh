/*
 * tc.cuh -- Blackwell (sm_100a/sm_103a) tensor-core helpers in inline PTX:
 * tcgen05 TMEM allocation, MMA issue and commit, TMEM loads, mbarriers
 * with bounded waits, and the shared-memory matrix descriptors of the
 * 128-byte-swizzled K-major layout.
 *
 * Layout used throughout: an operand tile of R rows x 64 K-elements
 * (16-bit) is R rows of 128 bytes; 8-row groups are 1024 bytes apart; in
 * row r the 16-byte chunk c is stored at chunk (c ^ (r & 7)).  The tile
 * starts on a 1024-byte boundary.  Descriptor: start address >> 4,
 * leading offset 1 (unused for this layout), stride offset 1024 >> 4,
 * descriptor version 1, layout type 2 (128-byte swizzle).  Moving 16
 * K-elements further adds 32 bytes to the start address.
 */
#pragma once

#include <stdint.h>

namespace zeta {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

/* byte offset of (row, 16-byte chunk) inside a 128B-swizzled tile */
__device__ __forceinline__ uint32_t sw128_offset(int row, int chunk) {
  return (uint32_t)((row >> 3) * 1024 + (row & 7) * 128 + ((chunk ^ (row & 7)) << 4));
}

__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);         /* start address */
  d |= (uint64_t)1 << 16;                          /* leading byte offset (unused) */
  d |= (uint64_t)((1024 >> 4) & 0x3FFF) << 32;     /* stride byte offset: 8 rows */
  d |= (uint64_t)1 << 46;                          /* descriptor version */
  d |= (uint64_t)2 << 61;                          /* 128-byte swizzle */
  return d;
}

/* instruction descriptor, kind::f16: D f32, A/B bf16 (1) or f16 (0),
 * both K-major, shape M x N */
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N, int ab_bf16) {
  return (1u << 4) | ((uint32_t)ab_bf16 << 7) | ((uint32_t)ab_bf16 << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}
/* instruction descriptor, kind::f8f6f4: D f32, A/B e4m3 (0), K-major */
__host__ __device__ constexpr uint32_t idesc_f8(int M, int N) {
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  /* make the initialised barrier visible to the async proxy (tcgen05.commit) */
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

/* bounded wait on an mbarrier phase; false when it gave up */
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t phase, uint32_t max_tries) {
  uint32_t ok = 0;
  for (uint32_t i = 0; i < max_tries; i++) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
    if (ok) return true;
    if (i > 64) __nanosleep(64);
  }
  return false;
}

/* plain arrival (the barrier counts its arrivals) */
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

/* arrive once and announce `bytes` of asynchronous transfers on `bar` */
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

/* TMA: a 2-D tile at (x = inner element, y = row) of the tensor map into
 * shared memory; completion is counted in bytes on `bar`.  x times the
 * element size must be a multiple of 16 bytes. */
__device__ __forceinline__ void tma_load_2d(void *dst, const void *tmap, int x, int y, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
      "[%4];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)tmap), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void prefetch_tmap(const void *tmap) {
  asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)tmap) : "memory");
}

/* generic-proxy shared-memory writes become visible to the tensor cores */
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

/* warp-collective TMEM allocation of `ncols` columns (power of 2 >= 32);
 * the address lands in *dst (shared memory) */
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

/* D[tmem] (+)= A[smem] x B[smem]^T, issued by one thread */
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_f8(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

/* arrive on `bar` when every MMA issued so far by this thread is done */
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

/* 16 consecutive 32-bit columns of this thread's TMEM lane */
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace zeta
