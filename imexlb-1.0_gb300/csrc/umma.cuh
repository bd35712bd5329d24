// Blackwell tensor-core primitives (sm_103a) as inline PTX: tensor memory
// (TMEM) allocation, tcgen05.mma with operands in shared memory, completion
// through an mbarrier, and reading the accumulator back.
//
// Operand layout in shared memory (no swizzle, K-major): an R x K bf16
// operand (R rows, K contiguous along a row in the GEMM sense) is cut into
// "core matrices" of 8 rows x 8 elements (8 x 16 bytes, 128 contiguous
// bytes, row stride 16 bytes). Core matrix (row group g, k chunk c) sits at
// byte (c * R/8 + g) * 128: the row groups of one k chunk are adjacent
// (stride 128 bytes, the descriptor's stride-dimension offset), k chunks are
// R/8 * 128 bytes apart (its leading-dimension offset). One MMA consumes a
// K slice of 16 elements (two k chunks).
#pragma once

#include <cstdint>

namespace imx {
namespace umma {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Element offset of (r, k) in the core-matrix layout of an operand with R rows.
__device__ __forceinline__ int cm_off(int r, int k, int R) {
  return (((k >> 3) * (R >> 3) + (r >> 3)) << 6) + ((r & 7) << 3) + (k & 7);
}

// Shared-memory matrix descriptor: start address, leading-dimension byte
// offset (between k chunks), stride-dimension byte offset (between row
// groups), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Descriptor of K slice s (16 elements) of an R-row operand at `base`.
__device__ __forceinline__ uint64_t slice_desc(uint32_t base, int R, int s) {
  const uint32_t kstride = (uint32_t)(R >> 3) * 128u;
  return smem_desc(base + (uint32_t)s * 2u * kstride, kstride, 128u);
}

// Instruction descriptor of kind::f16: bf16 A and B (both K-major), f32
// accumulator, shape M x N.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

// Warp-wide (all 32 lanes): allocate `ncols` TMEM columns (a power of two
// >= 32); the base address is written to *dst in shared memory.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_addr(dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

// Warp-wide: free the columns.
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Generic-proxy writes to shared memory become visible to the MMA.
__device__ __forceinline__ void fence_smem_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(1) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Bounded wait for phase `parity` of the barrier; false when it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int max_tries) {
  for (int i = 0; i < max_tries; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred q;\n\tmbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// One thread: D[tmem] (+)= A * B^T for a 128 x N x 16 slice.
__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, bool accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate ? 1u : 0u)
      : "memory");
}

// One thread: the barrier's phase completes when all MMAs issued so far have.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_addr(bar))
               : "memory");
}

// Warp-wide: 16 consecutive f32 columns of this warp's 32 TMEM lanes (lane i
// of the warp reads lane base+i); taddr = base | (lane base << 16) + column.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

}  // namespace umma
}  // namespace imx
