// 5th-generation tensor-core building blocks (tcgen05, sm_100a family) for
// the learned correction's BF16 contractions: shared-memory operand
// descriptors in the canonical no-swizzle K-major layout, the instruction
// descriptor of a BF16 x BF16 -> FP32 MMA, tensor-memory (TMEM) allocation,
// the single-thread MMA issue with its mbarrier commit, and the TMEM loads of
// the epilogue.  Written from the PTX ISA's description of tcgen05; every
// wait is bounded.
//
// Operand layout in shared memory (K-major, no swizzle): an R x K BF16 tile
// (R = M rows of A, or N rows of B) is a grid of 8 x 8 core matrices, each
// 8 rows of 16 contiguous bytes (128 bytes).  Element (r, k) lives at
//   (r / 8) * SBO + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2   bytes,
// SBO = K * 16: the core matrices of one 8-row group follow each other along
// K (leading byte offset, LBO = 128), the 8-row groups follow each other
// (stride byte offset, SBO).  One MMA consumes K = 16 (two core matrices
// along K); the next K step starts 256 bytes further.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace idfx {
namespace umma {

// byte offset of element (r, k) of a K-major no-swizzle tile with K columns
__host__ __device__ constexpr uint32_t kmajor_offset(int r, int k, int K) {
  return (uint32_t)((r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor: start address, LBO, SBO (all >> 4),
// descriptor version 1 (bits 46-47), base offset 0, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 (bits
// 17-22), M >> 4 (bits 24-28)
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// TMEM allocation of ncols columns (a power of two >= 32) by one whole warp;
// the base address is written to *slot (shared memory)
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// D[tmem] (+)= A[smem] . B[smem]^T, one thread
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// the mbarrier completes once every MMA this thread issued before has landed
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes made visible to the tensor core
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's TMEM lane (32x32b shape: warp
// w of the CTA reads lanes 32 (w % 4) .. + 31, thread t lane 32 (w % 4) + t)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void mbar_init1(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// at most `limit` try_wait attempts; false when it gave up
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, long long limit) {
  for (long long it = 0; it < limit; it++)
    if (mbar_test(bar, parity)) return true;
  return false;
}
constexpr long long kMmaSpin = 1ll << 22;

// A run of MMAs over K (multiple of 16): D (M x N, TMEM) (+)= A (M x K) . B
// (N x K)^T, both K-major no-swizzle tiles at a_base / b_base (shared
// addresses) with K columns; issued by one thread
__device__ __forceinline__ void mma_tile(uint32_t d_tmem, uint32_t a_base, uint32_t b_base, int K, uint32_t idesc,
                                         bool accumulate) {
  const uint32_t sbo = (uint32_t)K * 16u;
  for (int k = 0; k < K; k += 16) {
    const uint64_t ad = smem_desc(a_base + (uint32_t)k * 16u, 128u, sbo);
    const uint64_t bd = smem_desc(b_base + (uint32_t)k * 16u, 128u, sbo);
    mma_bf16(d_tmem, ad, bd, idesc, (accumulate || k > 0) ? 1u : 0u);
  }
}

}  // namespace umma
}  // namespace idfx
