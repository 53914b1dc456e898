/* Fifth-generation tensor-core (tcgen05) building blocks for sm_103a, written
 * as inline PTX: shared-memory operand layout and descriptors, the BF16 MMA
 * with FP32 accumulation in tensor memory (TMEM), commit to an mbarrier,
 * TMEM allocation and loads.
 *
 * Operand layout: K-major without swizzle.  A "core matrix" is 8 rows x 16
 * bytes (8 bf16 along K) stored as 128 contiguous bytes; core matrices follow
 * each other along K (leading-byte offset 128 B), then along M/N (stride-byte
 * offset K/8 * 128 B).  One MMA consumes K = 16, i.e. two core matrices along
 * K, so the next K step starts 256 B further.
 *
 * Accumulator layout for M = 128 (cta_group::1): row i of D is TMEM lane i,
 * column j is TMEM column base + j; warp w of a 4-warp group reads lanes
 * 32w .. 32w + 31.
 *
 * Every wait is bounded: a wait that gives up returns false, and the caller
 * records an error and skips the remaining tensor-core work of its tile. */
#pragma once

#include <cstdint>
#include <cuda_bf16.h>

namespace tc05 {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

/* Byte offset of element (r, k) in a K-major operand with K columns. */
__device__ __forceinline__ uint32_t kmaj(int r, int k, int K) {
  return (uint32_t)((((r >> 3) * (K >> 3) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}

/* Shared-memory matrix descriptor: start address, leading-byte offset (between
 * core matrices along K), stride-byte offset (between 8-row groups), descriptor
 * version 1, base offset 0, no swizzle. */
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

/* Instruction descriptor, kind::f16: D = FP32, A = B = BF16, both K-major,
 * dense, no negation; N >> 3 at bit 17, M >> 4 at bit 24. */
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

/* D[tmem] (+)= A * B^T, one instruction (K = 16), issued by one thread. */
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

/* A (M x K, K-major at a_saddr) times B (N x K, K-major at b_saddr)^T into
 * D at d_tmem: K/16 instructions.  Issued by one thread. */
__device__ __forceinline__ void gemm(uint32_t d_tmem, uint32_t a_saddr, uint32_t b_saddr, int M, int N, int K,
                                     bool accumulate) {
  const uint32_t id = idesc_bf16(M, N);
  const uint32_t sbo = (uint32_t)(K >> 3) << 7;
  for (int s = 0; s < (K >> 4); ++s)
    mma_bf16(d_tmem, sdesc(a_saddr + 256u * s, 128, sbo), sdesc(b_saddr + 256u * s, 128, sbo), id,
             (accumulate || s > 0) ? 1u : 0u);
}

/* Arrive on the mbarrier once every MMA issued so far by this thread is done. */
__device__ __forceinline__ void commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
/* Generic-proxy shared-memory writes become visible to the tensor core. */
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

/* Bounded wait for the phase with the given parity: gives up after about
 * 2^31 SM cycles (about a second). */
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > (1ll << 31)) return false;
  return true;
}

/* TMEM allocation by one whole warp; the base address lands in *slot. */
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

/* 16 consecutive FP32 columns of this thread's lane (warp-collective).  The
 * load is asynchronous: its destination registers are valid only after
 * tcgen05.wait::ld, so both are one asm statement and the compiler cannot
 * move a use of the registers above the wait. */
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

/* TMEM address of (lane, column) relative to an allocation base. */
__device__ __forceinline__ uint32_t taddr(uint32_t base, int lane, int col) {
  return base + ((uint32_t)lane << 16) + (uint32_t)col;
}

__device__ __forceinline__ uint16_t bf16_bits(float x) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(x));
}

/* Eight bf16 (one 16-byte row of a core matrix) from eight floats. */
__device__ __forceinline__ uint4 pack8(const float* x) {
  uint4 u;
  u.x = (uint32_t)bf16_bits(x[0]) | ((uint32_t)bf16_bits(x[1]) << 16);
  u.y = (uint32_t)bf16_bits(x[2]) | ((uint32_t)bf16_bits(x[3]) << 16);
  u.z = (uint32_t)bf16_bits(x[4]) | ((uint32_t)bf16_bits(x[5]) << 16);
  u.w = (uint32_t)bf16_bits(x[6]) | ((uint32_t)bf16_bits(x[7]) << 16);
  return u;
}

}  // namespace tc05
