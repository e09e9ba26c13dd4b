// Fifth-generation tensor cores (tcgen05) for the dense small-dimension bucket:
// shared-memory operand descriptors, the TF32 instruction descriptor, tensor-memory
// (TMEM) allocation, MMA issue / commit and accumulator loads, as inline PTX.
//
// Operand layout (K-major, no swizzle): a tile of R rows x K columns of 32-bit values is
// stored as 8-row x 16-byte "core matrices"; element (r, k) sits at
//   (r / 8) * SBO + (k / 4) * 128 + (r % 8) * 16 + (k % 4) * 4   bytes,
// so the core matrices of one 8-row band are adjacent along K (leading-dimension byte
// offset 128) and bands are SBO = 32 * K bytes apart (stride-dimension byte offset).
// One MMA of kind::tf32 consumes K = 8 (two core matrices along K); the next K step starts
// 256 bytes further.
#pragma once
#include <stdint.h>

#include "common.cuh"

namespace qg {
namespace tc {

constexpr uint32_t LBO = 128;  // bytes between core matrices along K

__device__ __forceinline__ uint32_t band_bytes(int k_cols) { return 32u * (uint32_t)k_cols; }

// byte offset of element (r, k) in a K-major tile with k_cols columns
__device__ __forceinline__ uint32_t core_off(int r, int k, int k_cols) {
  return (uint32_t)(r >> 3) * band_bytes(k_cols) + (uint32_t)(k >> 2) * LBO +
         (uint32_t)(r & 7) * 16u + (uint32_t)(k & 3) * 4u;
}

// Shared-memory matrix descriptor: start address, leading- and stride-dimension byte
// offsets (in 16-byte units), the descriptor version 1 of this tensor-core generation
// (bits 46-47) and swizzle mode 0 (none, bits 61-63).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::tf32: FP32 accumulator (bits 4-5 = 1), A and B in TF32
// (bits 7-9, 10-12 = 2), optional negation of A (bit 13), both operands K-major (bits 15,
// 16 = 0), N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N, bool neg_a) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((neg_a ? 1u : 0u) << 13) |
         ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy writes of shared memory made visible to the tensor cores' async proxy
__device__ __forceinline__ void fence_smem_to_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// one warp: allocate ncols (a power of two, 32..512) TMEM columns; the address lands in
// *dst (shared memory)
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
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

// D (+)= A B^T for the operands described by adesc / bdesc; issued by one thread
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, bool accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate ? 1u : 0u)
      : "memory");
}
// the completion of every MMA issued so far by this thread arrives on the mbarrier
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// 8 consecutive FP32 columns of this thread's TMEM lane (warp w reads lanes 32 (w % 4) ...)
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// x as a TF32 pair: hi keeps the 10 explicit mantissa bits of TF32 (rounded), lo = x - hi
// is exact in FP32; hi*y_hi + hi*y_lo + lo*y_hi then carries about FP32 precision
// ("3xTF32", Markidis et al. 2018 for the FP16 form of the split).
__device__ __forceinline__ void tf32_split(float x, float& hi, float& lo) {
  uint32_t u = __float_as_uint(x);
  u = (u + 0x1000u) & 0xFFFFE000u;  // round the mantissa to 10 bits (ties away)
  hi = __uint_as_float(u);
  lo = x - hi;
}

}  // namespace tc
}  // namespace qg
