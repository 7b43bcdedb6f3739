// Shared helpers of the tcgen05 kernels (sm_103a): shared-memory matrix descriptors in the K-major canonical layout
// without swizzle, the kind::f16 instruction descriptor, the MMA issue, bounded mbarrier waits and the bfloat16 split
// of float32 values.
#pragma once

#include "common.cuh"

namespace citrus {

constexpr int kTcM = 128;                         // MMA rows of every tcgen05 kernel here
constexpr uint64_t kTcTimeoutNs = 1000000000ull;  // bound of every wait for the tensor cores

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// bf16 bits of x, round to nearest even (finite inputs)
__device__ __forceinline__ uint32_t bf16_bits(float x) {
  const uint32_t u = __float_as_uint(x);
  return (u + 0x7FFFu + ((u >> 16) & 1u)) >> 16;
}

__device__ __forceinline__ void split_pair(float x0, float x1, uint32_t& hi, uint32_t& lo) {
  const uint32_t h0 = bf16_bits(x0), h1 = bf16_bits(x1);
  const float r0 = x0 - __uint_as_float(h0 << 16), r1 = x1 - __uint_as_float(h1 << 16);
  hi = h0 | (h1 << 16);
  lo = bf16_bits(r0) | (bf16_bits(r1) << 16);
}

// Shared-memory matrix descriptor, K-major, no swizzle: start address, leading byte offset (between core matrices
// adjacent in K), stride byte offset (between 8-row groups), the descriptor version bit of this architecture.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
  d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
  d |= (uint64_t)1 << 46;
  return d;  // base offset 0, swizzle none
}

// Instruction descriptor of kind::f16: bf16 A and B, float32 accumulator, both K-major, M = 128 and N columns.
__host__ __device__ constexpr uint32_t idesc_bf16(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kTcM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, uint64_t t0) {
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
    if (global_timer_ns() - t0 > kTcTimeoutNs) return false;
  }
}

// Core-matrix byte offset of element row r (M or N index), column k (K index) inside one 16-wide K step region.
__device__ __forceinline__ uint32_t core_offset(int r, int k) {
  return (uint32_t)((((r >> 3) * 2 + (k >> 3)) * 128) + (r & 7) * 16 + (k & 7) * 2);
}

}  // namespace citrus
