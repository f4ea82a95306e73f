// sg_af_mma.cuh -- building blocks of the learned filter's tensor-core
// kernels: the activation, shared-memory staging of BF16 operand tiles and
// one layer's MMA chain (M = 128 rows, one issuing thread, bounded wait).
#pragma once

#include "sg_learned.cuh"
#include "sg_tc.cuh"

namespace sg {

// GELU in its tanh form (Hendrycks and Gimpel, "Gaussian Error Linear Units",
// 2016): 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))), with the hardware
// tanh (tanh.approx).  The forward pass evaluates it in packed BF16
// (gelu_bf16x2); the backward pass takes its derivative in FP32.
constexpr float GELU_K0 = 0.7978845608028654f;            // sqrt(2 / pi)
constexpr float GELU_K1 = 0.7978845608028654f * 0.044715f;
__device__ inline float tanh_hw(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ inline float gelu_grad(float x) {
  float const x2 = x * x;
  float const t = tanh_hw(x * (GELU_K0 + GELU_K1 * x2));
  return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * (GELU_K0 + 3.0f * GELU_K1 * x2);
}

// GELU of two pre-activations, evaluated in packed BF16 arithmetic (the
// activations are BF16 operands of the next layer): returns the BF16 pair
// as the low and high halves of a 32-bit word.
__device__ inline uint32_t gelu_bf16x2(float a, float b) {
  __nv_bfloat162 const x = __floats2bfloat162_rn(a, b);
  __nv_bfloat162 const k0 = __float2bfloat162_rn(GELU_K0), k1 = __float2bfloat162_rn(GELU_K1);
  __nv_bfloat162 const u = __hmul2(x, __hfma2(__hmul2(x, x), k1, k0));
  uint32_t t;
  asm("tanh.approx.bf16x2 %0, %1;" : "=r"(t) : "r"(*reinterpret_cast<uint32_t const*>(&u)));
  __nv_bfloat162 const h = __hmul2(x, __float2bfloat162_rn(0.5f));
  __nv_bfloat162 const g = __hfma2(h, *reinterpret_cast<__nv_bfloat162 const*>(&t), h);
  return *reinterpret_cast<uint32_t const*>(&g);
}

// GELU of 16 pre-activations v + bias into a row of a K-major tile (columns
// k .. k + 15); `out` (optional) receives the activations as floats.
__device__ inline void gelu_row16(uint8_t* tile, uint32_t row, uint32_t k, uint32_t K, float const* v,
                                  float const* bias, float* out = nullptr) {
  uint32_t w[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) w[i] = gelu_bf16x2(v[2 * i] + bias[2 * i], v[2 * i + 1] + bias[2 * i + 1]);
  *reinterpret_cast<uint4*>(tile + tile_off(row, k, K)) = make_uint4(w[0], w[1], w[2], w[3]);
  *reinterpret_cast<uint4*>(tile + tile_off(row, k + 8, K)) = make_uint4(w[4], w[5], w[6], w[7]);
  if (out) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      out[2 * i] = __uint_as_float(w[i] << 16);
      out[2 * i + 1] = __uint_as_float(w[i] & 0xFFFF0000u);
    }
  }
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
