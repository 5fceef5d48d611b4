// fedg_umma.cuh -- helpers of the kernels that issue 5th-generation tensor-core MMAs (tcgen05):
// shared-memory matrix descriptors, bounded mbarrier waits.
#pragma once
#include <cstdint>

namespace fedg {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor of a K-major operand in the no-swizzle canonical layout: 8-row x
// 16-byte core matrices, K-adjacent core matrices lbo bytes apart, 8-row groups sbo bytes apart.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
         (1ull << 46);  // descriptor version 1, base offset 0, no swizzle
}

// Instruction descriptor of tcgen05.mma kind::f16: FP32 accumulator, BF16 A and B, both K-major,
// M x N tile.
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Instruction descriptor of tcgen05.mma kind::tf32: FP32 accumulator, TF32 A and B (format 2), both
// K-major, M x N tile.
__host__ __device__ constexpr uint32_t umma_idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// polls of a drain wait, and the default limit of the normal-path waits
constexpr int DRAIN_POLLS = 1 << 20;

// Waits for the phase of `parity` of an mbarrier, polling at most `limit` times; false on expiry.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t mbar, uint32_t parity, int limit) {
  for (int it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

}  // namespace fedg
