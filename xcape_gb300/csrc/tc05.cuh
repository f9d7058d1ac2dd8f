// tc05.cuh -- the 5th-generation tensor-core path of sm_103a in inline PTX:
// tensor-memory (TMEM) allocation, tcgen05.mma with both operands in shared
// memory, its completion through an mbarrier, and tcgen05.ld of the FP32
// accumulator.  Used by the network training kernel (guess_mlp.cu).
//
// Operand tiles live in shared memory in the canonical K-major layout
// without swizzle: the tile is cut into core matrices of 8 rows x 16 bytes
// (8 BF16 elements of K), each stored as 128 contiguous bytes; core matrix
// (i, j) -- rows 8i .. 8i + 7, K elements 8j .. 8j + 7 -- starts at byte
// (i * (K / 8) + j) * 128.  In the shared-memory descriptor the leading
// byte offset (LBO) is then the step between core matrices along K, 128 B,
// and the stride byte offset (SBO) the step between 8-row groups,
// K / 8 * 128 B.  One kind::f16 MMA consumes K = 16 (two core matrices
// along K), so the k-th MMA of a product starts 256 B * k into the tiles.
//
// The accumulator D of an M = 128 MMA with cta_group::1 holds row i in TMEM
// lane i and column j in TMEM column (base + j); warp w of the CTA may read
// lanes 32 (w % 4) .. 32 (w % 4) + 31 only.
#pragma once

#include <stdint.h>

namespace xc {
namespace tc05 {

// Element offset of (row r, k) in a canonical K-major tile of K columns.
__host__ __device__ __forceinline__ int canon(int r, int k, int K) {
  return (((r >> 3) * (K >> 3) + (k >> 3)) << 6) + ((r & 7) << 3) + (k & 7);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: start address, LBO and SBO (bytes,
// multiples of 16), version 1 (tcgen05), no swizzle.
__device__ __forceinline__ uint64_t sdesc(const void *tile, uint32_t lbo, uint32_t sbo) {
  const uint64_t a = (uint64_t)((smem_u32(tile) >> 4) & 0x3FFFu);
  return a | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) | ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) |
         ((uint64_t)1 << 46);
}

// Instruction descriptor of kind::f16 with BF16 A and B (both K-major) and
// an FP32 accumulator, for an M x N product.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4)                      // D format: F32
         | (1u << 7)                    // A format: BF16
         | (1u << 10)                   // B format: BF16
         | ((uint32_t)(N >> 3) << 17)   // N / 8
         | ((uint32_t)(M >> 4) << 24);  // M / 16
}

// Allocates `ncols` TMEM columns (a power of two, 32 .. 512) for the CTA and
// writes their base address to *dst (shared memory).  One whole warp calls
// it; the same warp must free them (tmem_free).
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n"
               :: "r"(smem_u32(dst)), "r"(ncols) : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n"
               :: "r"(taddr), "r"(ncols) : "memory");
}

// D (TMEM) = A B^T (+ D when `accumulate`), issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
      :: "r"(d_tmem), "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate) : "memory");
}

// The mbarrier arrives once every MMA this thread issued before has completed.
__device__ __forceinline__ void commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n"
               :: "r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}
// Makes this thread's generic-proxy shared-memory writes visible to the
// tensor cores (the async proxy).
__device__ __forceinline__ void fence_smem_async() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" :: "r"(smem_u32(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

// Waits for the mbarrier phase with parity `phase` to complete, at most
// `limit` polls (each poll may itself suspend for a while); false if the
// limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t phase, uint32_t limit) {
  const uint32_t a = smem_u32(bar);
  for (uint32_t it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done) : "r"(a), "r"(phase) : "memory");
    if (done) return true;
  }
  return false;
}

// 16 consecutive FP32 columns of this thread's TMEM lane, from `taddr`
// (lane field = the warp's first lane).  The wait for the load is in the
// same asm statement, so no use of the registers can be scheduled before it.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

}  // namespace tc05
}  // namespace xc
