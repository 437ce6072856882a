// tcgen05 (5th-generation tensor core) helpers for sm_103a, in inline PTX.
//
// Used by the mixed-precision contractions: one elected thread issues
// tcgen05.mma.kind::tf32 or kind::f16 (BF16 operands) with both operands in
// shared memory (K-major, 128-byte swizzle) and the FP32 accumulator in
// tensor memory (TMEM);
// completion is tracked with mbarriers through tcgen05.commit; the epilogue
// reads TMEM with tcgen05.ld.  Every wait is bounded: on expiry the caller
// records an error and leaves the loop instead of spinning forever.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace occx {
namespace umma {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---- mbarrier --------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile("{\n\t.reg .pred p;\n\t"
               "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
               "selp.u32 %0, 1, 0, p;\n\t}"
               : "=r"(ok)
               : "r"(smem_u32(bar)), "r"(parity)
               : "memory");
  return ok != 0;
}
// Bounded wait for the phase with the given parity to complete.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t max_iter) {
  for (uint32_t i = 0; i < max_iter; i++)
    if (mbar_try_wait(bar, parity))
      return true;
  return false;
}

// Plain arrive (count 1) by this thread.
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// Arrive and add `bytes` to the transaction count the phase waits for.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// ---- TMA -------------------------------------------------------------------
// 2D tiled bulk tensor load global -> shared, completion counted in bytes on
// `bar`.  x is the innermost coordinate (elements; x * element size must be a
// multiple of 16 bytes), y the row.
__device__ __forceinline__ void tma_load_2d(void *dst, const void *tmap, int x, int y,
                                            uint64_t *bar) {
  asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
               " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
               "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(smem_u32(bar))
               : "memory");
}
// Plain (non-tensor) bulk copy global -> shared of `bytes` (multiple of 16;
// both addresses 16-byte aligned), completion counted in bytes on `bar`.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes,
                                          uint64_t *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes"
               " [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
               "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tma_prefetch_desc(const void *tmap) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(tmap)) : "memory");
}

// ---- fences ----------------------------------------------------------------
// generic-proxy shared-memory writes -> visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// ---- tensor memory ---------------------------------------------------------
// Executed by one full warp; writes the TMEM base address to *dst.
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

// 32 lanes x 32 bits, 16 consecutive columns starting at taddr.  The warp
// reads its own 32-lane quarter of TMEM (lane field of taddr).  The load is
// warp-collective (.sync.aligned): every lane must execute it together, so
// the warp is reconverged first (its lanes may leave a preceding mbarrier
// poll in different iterations).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  __syncwarp();
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
               "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                 "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
                 "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
               : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() {
  __syncwarp();
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// ---- MMA -------------------------------------------------------------------
// Shared-memory matrix descriptor, K-major operand with the 128-byte swizzle:
// rows of 128 bytes (32 TF32 values), 8-row core groups 1024 bytes apart,
// tile base 1024-byte aligned.  Advancing K by 8 TF32 values inside the
// 128-byte row is done by adding 32 bytes to the start address.
__device__ __forceinline__ uint64_t desc_kmajor_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);  // start address
  d |= static_cast<uint64_t>(1) << 16;                   // leading byte offset (unused here)
  d |= static_cast<uint64_t>(1024 >> 4) << 32;           // stride byte offset: 8 rows
  d |= static_cast<uint64_t>(1) << 46;                   // descriptor version (tcgen05)
  d |= static_cast<uint64_t>(2) << 61;                   // 128-byte swizzle
  return d;
}

// Instruction descriptor: kind::tf32, FP32 accumulate, A and B TF32 and
// K-major, shape M x N.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4)                                   // D format F32
         | (2u << 7)                                 // A format TF32
         | (2u << 10)                                // B format TF32
         | (static_cast<uint32_t>(N >> 3) << 17)     // N / 8
         | (static_cast<uint32_t>(M >> 4) << 24);    // M / 16
}

// Instruction descriptor: kind::f16 with BF16 A and B (K-major), FP32
// accumulate, shape M x N.  One MMA covers K = 16 (32 bytes of a row), the
// same bytes per step as a TF32 MMA's K = 8, so the 128-byte-swizzled tile
// layout and its descriptors are shared with the TF32 path.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4)                                   // D format F32
         | (1u << 7)                                 // A format BF16
         | (1u << 10)                                // B format BF16
         | (static_cast<uint32_t>(N >> 3) << 17)     // N / 8
         | (static_cast<uint32_t>(M >> 4) << 24);    // M / 16
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile("{\n\t.reg .pred p;\n\t"
               "setp.ne.b32 p, %4, 0;\n\t"
               "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
               "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
               : "memory");
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile("{\n\t.reg .pred p;\n\t"
               "setp.ne.b32 p, %4, 0;\n\t"
               "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
               "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
               : "memory");
}

// Arrive on the mbarrier once all previously issued MMAs of this thread finish.
__device__ __forceinline__ void commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

// ---- TF32 split --------------------------------------------------------------
// x = hi + lo with hi, lo TF32 (round-to-nearest); hi*hi + hi*lo + lo*hi keeps
// about FP32 accuracy ("3xTF32").
__device__ __forceinline__ void split_tf32(float x, uint32_t &hi, uint32_t &lo) {
  uint32_t h, l;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
  float r = x - __uint_as_float(h);
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(r));
  hi = h;
  lo = l;
}

// Byte offset of 16-byte chunk c (0..7) of row r in a K-major 128B-swizzled tile.
__device__ __forceinline__ uint32_t sw128_offset(uint32_t r, uint32_t c) {
  return (r >> 3) * 1024u + (r & 7u) * 128u + ((c ^ (r & 7u)) << 4);
}

} // namespace umma
} // namespace occx
