// sg_af_mma.cuh -- building blocks of the learned filter's tensor-core
// kernels: the activation, shared-memory staging of BF16 operand tiles and
// one layer's MMA chain (M = 128 rows, one issuing thread, bounded wait).
#pragma once

#include "sg_learned.cuh"
#include "sg_tc.cuh"

namespace sg {

// GELU in its tanh form (Hendrycks and Gimpel, "Gaussian Error Linear Units",
// 2016): 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))), with the hardware
// tanh (tanh.approx.f32, about 2^-11 relative error) -- the activations are
// rounded to BF16 (2^-9) for the next layer in any case.
constexpr float GELU_K0 = 0.7978845608028654f;            // sqrt(2 / pi)
constexpr float GELU_K1 = 0.7978845608028654f * 0.044715f;
__device__ inline float tanh_hw(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ inline float gelu(float x) {
  float const t = tanh_hw(x * (GELU_K0 + GELU_K1 * (x * x)));
  float const h = 0.5f * x;
  return h + h * t;
}
__device__ inline float gelu_grad(float x) {
  float const x2 = x * x;
  float const t = tanh_hw(x * (GELU_K0 + GELU_K1 * x2));
  return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * (GELU_K0 + 3.0f * GELU_K1 * x2);
}

// Copies `bytes` (multiple of 16) from global to shared memory.
__device__ inline void copy16(void* dst, void const* src, int bytes) {
  for (int i = threadIdx.x; i < bytes / 16; i += blockDim.x)
    reinterpret_cast<uint4*>(dst)[i] = reinterpret_cast<uint4 const*>(src)[i];
}

// Writes 8 consecutive values (k .. k + 7, k a multiple of 8) of a row as
// BF16 into a K-major core-matrix tile with K columns.
__device__ inline void put8(uint8_t* tile, uint32_t row, uint32_t k, uint32_t K, float const* v) {
  uint4 u;
  uint32_t* w = &u.x;
#pragma unroll
  for (int i = 0; i < 4; ++i) w[i] = static_cast<uint32_t>(bf16_bits(v[2 * i])) | (static_cast<uint32_t>(bf16_bits(v[2 * i + 1])) << 16);
  *reinterpret_cast<uint4*>(tile + tile_off(row, k, K)) = u;
}

// TMEM address of this thread's row (lane) at column `col`
__device__ inline uint32_t lane_addr(uint32_t base, uint32_t col) {
  return base + ((threadIdx.x & ~31u) << 16) + col;
}

// Layer l: D[tmem col] = A (tile, K columns) x B^T (weights image, N rows),
// issued by thread 0; every thread waits for completion.
__device__ inline bool layer_mma(uint32_t d, uint8_t const* a, uint8_t const* b, uint32_t K, uint32_t N, uint32_t acc,
                                 uint64_t* bar, uint32_t& phase) {
  if (threadIdx.x == 0) {
    tc_fence_after();
    for (uint32_t ks = 0; ks < K / 16; ++ks)
      mma_bf16(d, tile_desc(a, K, ks), tile_desc(b, K, ks), idesc_bf16(AF_TILE, N), (ks > 0 || acc) ? 1u : 0u);
    mma_commit(bar);
  }
  bool ok = mbar_wait(bar, phase);
  phase ^= 1u;
  tc_fence_after();
  return ok;
}

}  // namespace sg
