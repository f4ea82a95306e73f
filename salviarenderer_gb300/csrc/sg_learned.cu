// sg_learned.cu -- tensor-core kernels of the learned anisotropic filter:
// weight packing, inference (k_af_infer), training steps (k_af_train) and
// the Adam update (k_af_adam).  Every matrix product runs on tcgen05.mma
// with BF16 operands in shared memory and FP32 accumulators in tensor
// memory; one thread issues the MMAs, all 128 threads of the CTA move data.
#include <cuda_runtime.h>

#include "sg_af_mma.cuh"

namespace sg {

// Writes the BF16 operand images of the current fp32 parameters.
__global__ void k_af_pack(AfModelDev M) {
  uint16_t* img = reinterpret_cast<uint16_t*>(M.img);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < AF_IMG_BYTES / 2; i += gridDim.x * blockDim.x)
    img[i] = 0;
  __syncthreads();
  // (a single CTA runs this kernel, so the zeroing above completes first)
  float const* P = M.params;
  for (int i = threadIdx.x; i < AF_H * AF_K1; i += blockDim.x) {  // W1 [64 x 32]
    int o = i / AF_K1, k = i % AF_K1;
    float w = k < AF_F ? P[AF_OFF_W1 + o * AF_F + k] : 0.0f;
    img[(AF_IMG_W1 + tile_off(o, k, AF_K1)) / 2] = bf16_bits(w);
  }
  for (int i = threadIdx.x; i < AF_H * AF_H; i += blockDim.x) {  // W2 [64 x 64] and W2^T
    int o = i / AF_H, k = i % AF_H;
    uint16_t w = bf16_bits(P[AF_OFF_W2 + o * AF_H + k]);
    img[(AF_IMG_W2 + tile_off(o, k, AF_H)) / 2] = w;
    img[(AF_IMG_W2T + tile_off(k, o, AF_H)) / 2] = w;
  }
  for (int i = threadIdx.x; i < AF_N3 * AF_H; i += blockDim.x) {  // W3 [16 x 64] and W3^T [64 x 16]
    int o = i / AF_H, k = i % AF_H;
    uint16_t w = o < AF_O ? bf16_bits(P[AF_OFF_W3 + o * AF_H + k]) : 0;
    img[(AF_IMG_W3 + tile_off(o, k, AF_H)) / 2] = w;
    img[(AF_IMG_W3T + tile_off(k, o, AF_N3)) / 2] = w;
  }
}

// Inference: rows of 32 BF16 features -> 8 floats per row (RGBA, confidence
// as a probability, 3 unused); `skip` (fp32 tap means, one float4 per row)
// is added to the colour.  One CTA per SM walks tiles of 128 rows.
struct InferSmem {
  uint8_t w1[AF_H * AF_K1 * 2], w2[AF_H * AF_H * 2], w3[AF_N3 * AF_H * 2];
  uint8_t x[AF_TILE * AF_K1 * 2], h1[AF_TILE * AF_H * 2], h2[AF_TILE * AF_H * 2];
  float b1[AF_H], b2[AF_H], b3[AF_N3];
  uint64_t bar;
  uint32_t tmem;
};

__global__ void __launch_bounds__(AF_TILE, 1) k_af_infer(AfModelDev M, uint16_t const* X, float4 const* skip,
                                                          uint32_t n, float* out, unsigned int* status) {
  extern __shared__ __align__(128) uint8_t smem_raw[];
  InferSmem& s = *reinterpret_cast<InferSmem*>(smem_raw);
  uint32_t const tid = threadIdx.x;
  if (tid < 32) tmem_alloc(&s.tmem, 256);
  if (tid == 0) mbar_init(&s.bar, 1);
  copy16(s.w1, M.img + AF_IMG_W1, sizeof(s.w1));
  copy16(s.w2, M.img + AF_IMG_W2, sizeof(s.w2));
  copy16(s.w3, M.img + AF_IMG_W3, sizeof(s.w3));
  for (uint32_t i = tid; i < AF_H; i += blockDim.x) {
    s.b1[i] = M.params[AF_OFF_B1 + i];
    s.b2[i] = M.params[AF_OFF_B2 + i];
  }
  if (tid < AF_N3) s.b3[tid] = tid < AF_O ? M.params[AF_OFF_B3 + tid] : 0.0f;
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  uint32_t const tm = s.tmem;
  uint32_t phase = 0;
  bool ok = true;
  for (uint32_t t0 = blockIdx.x * AF_TILE; t0 < n && ok; t0 += gridDim.x * AF_TILE) {
    uint32_t const row = t0 + tid;
    // features of this row into the A tile
    uint4 const* src = reinterpret_cast<uint4 const*>(X + static_cast<size_t>(row) * AF_K1);
#pragma unroll
    for (int j = 0; j < AF_K1 / 8; ++j) {
      uint4 v = row < n ? src[j] : make_uint4(0, 0, 0, 0);
      *reinterpret_cast<uint4*>(s.x + tile_off(tid, 8 * j, AF_K1)) = v;
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    ok = ok && layer_mma(tm, s.x, s.w1, AF_K1, AF_H, 0, &s.bar, phase);
    float v[16];
#pragma unroll
    for (int c = 0; c < AF_H; c += 16) {
      tmem_ld16(lane_addr(tm, c), v);
      gelu_row16(s.h1, tid, c, AF_H, v, s.b1 + c);
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    ok = ok && layer_mma(tm + 64, s.h1, s.w2, AF_H, AF_H, 0, &s.bar, phase);
#pragma unroll
    for (int c = 0; c < AF_H; c += 16) {
      tmem_ld16(lane_addr(tm, 64 + c), v);
      gelu_row16(s.h2, tid, c, AF_H, v, s.b2 + c);
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    ok = ok && layer_mma(tm + 128, s.h2, s.w3, AF_H, AF_N3, 0, &s.bar, phase);
    tmem_ld16(lane_addr(tm, 128), v);
    if (row < n) {
      float4* o = reinterpret_cast<float4*>(out + static_cast<size_t>(row) * 8);
      float4 const k = skip[row];
      o[0] = make_float4(k.x + (v[0] + s.b3[0]), k.y + (v[1] + s.b3[1]), k.z + (v[2] + s.b3[2]),
                         k.w + (v[3] + s.b3[3]));
      o[1] = make_float4(1.0f / (1.0f + expf(-(v[4] + s.b3[4]))), 0.0f, 0.0f, 0.0f);
    }
    tc_fence_before();
    __syncthreads();
  }
  if (!ok && tid == 0) atomicOr(status, 1u);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (tid < 32) tmem_dealloc(tm, 256);
}

// ---------------------------------------------------------------------------
// Training: forward and backward of tiles of 128 samples on the tensor cores.
//
// Activation products are M = 128 (samples) x N x K: D1 = X W1^T,
// D2 = H1 W2^T, D3 = H2 W3^T, dH2 = dOut W3, dH1 = dH2pre W2.  Weight
// gradients are M = 128 x N x K = 128 (samples) with the activations
// transposed into the A operand and accumulated in tensor memory over every
// tile the CTA takes: G1 = [H1^T; H2^T] [dH2pre^T; dOut^T]^T (the diagonal
// blocks are dW2^T and dW3^T), G2 = [X^T; 1] dH1pre (dW1^T and, in the
// row of ones, db1), G3 = [X^T; 1] [dH2pre^T; dOut^T]^T (db2, db3 in the row
// of ones).  Loss per sample: squared colour error plus the binary
// cross-entropy of the confidence against exp(-AF_CONF_K * max |error|).
constexpr float AF_CONF_K = 32.0f;
constexpr int AF_ONES_ROW = 32;  // the row of ones in the transposed input tile
// tensor-memory columns
constexpr uint32_t TM_D1 = 0, TM_D2 = 64, TM_D3 = 128, TM_DH2 = 144, TM_DH1 = 208, TM_G1 = 272, TM_G2 = 352,
                   TM_G3 = 416;

struct TrainSmem {
  uint8_t w1[AF_H * AF_K1 * 2], w2[AF_H * AF_H * 2], w3[AF_N3 * AF_H * 2], w3t[AF_H * AF_N3 * 2],
      w2t[AF_H * AF_H * 2];
  uint8_t x[AF_TILE * AF_K1 * 2], h1[AF_TILE * AF_H * 2], h2[AF_TILE * AF_H * 2], dout[AF_TILE * AF_N3 * 2],
      dh2[AF_TILE * AF_H * 2];
  // K = 128 (samples) operands of the weight gradients
  uint8_t a1[128 * AF_TILE * 2], a2[128 * AF_TILE * 2], bt1[80 * AF_TILE * 2], bt2[64 * AF_TILE * 2];
  float b1[AF_H], b2[AF_H], b3[AF_N3];
  float loss;
  uint64_t bar;
  uint32_t tmem;
};

// element (row, col) of a K = 128 tile, as BF16
__device__ inline void put_t(uint8_t* tile, uint32_t row, uint32_t col, float v) {
  *reinterpret_cast<uint16_t*>(tile + tile_off(row, col, AF_TILE)) = bf16_bits(v);
}

__global__ void __launch_bounds__(AF_TILE, 1) k_af_train(AfModelDev M, uint16_t const* X, float4 const* Y,
                                                          uint32_t n, float inv_batch, float* loss_out,
                                                          unsigned int* status) {
  extern __shared__ __align__(128) uint8_t smem_raw[];
  TrainSmem& s = *reinterpret_cast<TrainSmem*>(smem_raw);
  uint32_t const tid = threadIdx.x;
  if (tid < 32) tmem_alloc(&s.tmem, 512);
  if (tid == 0) {
    mbar_init(&s.bar, 1);
    s.loss = 0.0f;
  }
  copy16(s.w1, M.img + AF_IMG_W1, sizeof(s.w1));
  copy16(s.w2, M.img + AF_IMG_W2, sizeof(s.w2));
  copy16(s.w3, M.img + AF_IMG_W3, sizeof(s.w3));
  copy16(s.w3t, M.img + AF_IMG_W3T, sizeof(s.w3t));
  copy16(s.w2t, M.img + AF_IMG_W2T, sizeof(s.w2t));
  for (uint32_t i = tid; i < sizeof(s.a2) / 16; i += blockDim.x) reinterpret_cast<uint4*>(s.a2)[i] = make_uint4(0, 0, 0, 0);
  for (uint32_t i = tid; i < AF_H; i += blockDim.x) {
    s.b1[i] = M.params[AF_OFF_B1 + i];
    s.b2[i] = M.params[AF_OFF_B2 + i];
  }
  if (tid < AF_N3) s.b3[tid] = tid < AF_O ? M.params[AF_OFF_B3 + tid] : 0.0f;
  __syncthreads();
  put_t(s.a2, AF_ONES_ROW, tid, 1.0f);  // the row of ones (sums over the tile's samples)
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  uint32_t const tm = s.tmem;
  uint32_t phase = 0;
  bool ok = true, any = false;
  float lsum = 0.0f;
  for (uint32_t t0 = blockIdx.x * AF_TILE; t0 < n && ok; t0 += gridDim.x * AF_TILE) {
    uint32_t const row = t0 + tid;
    bool const valid = row < n;
    // inputs: the A tile of layer 1 and, transposed, rows 0..23 of a2
    uint4 const* src = reinterpret_cast<uint4 const*>(X + static_cast<size_t>(row) * AF_K1);
#pragma unroll
    for (int j = 0; j < AF_K1 / 8; ++j) {
      uint4 v = valid ? src[j] : make_uint4(0, 0, 0, 0);
      *reinterpret_cast<uint4*>(s.x + tile_off(tid, 8 * j, AF_K1)) = v;
      uint32_t const w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        int const k = 8 * j + q;
        if (k < AF_F)
          *reinterpret_cast<uint16_t*>(s.a2 + tile_off(k, tid, AF_TILE)) = static_cast<uint16_t>(w[q >> 1] >> (16 * (q & 1)));
      }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    ok = ok && layer_mma(tm + TM_D1, s.x, s.w1, AF_K1, AF_H, 0, &s.bar, phase);
    float v[16];
#pragma unroll
    for (int c = 0; c < AF_H; c += 16) {
      tmem_ld16(lane_addr(tm, TM_D1 + c), v);
      gelu_row16(s.h1, tid, c, AF_H, v, s.b1 + c, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) put_t(s.a1, c + i, tid, v[i]);
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    ok = ok && layer_mma(tm + TM_D2, s.h1, s.w2, AF_H, AF_H, 0, &s.bar, phase);
#pragma unroll
    for (int c = 0; c < AF_H; c += 16) {
      tmem_ld16(lane_addr(tm, TM_D2 + c), v);
      gelu_row16(s.h2, tid, c, AF_H, v, s.b2 + c, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) put_t(s.a1, 64 + c + i, tid, v[i]);
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    ok = ok && layer_mma(tm + TM_D3, s.h2, s.w3, AF_H, AF_N3, 0, &s.bar, phase);
    // loss and its gradient with respect to the outputs
    tmem_ld16(lane_addr(tm, TM_D3), v);
    float d[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) d[i] = 0.0f;
    if (valid) {
      float4 const y = Y[row];
      float const yy[4] = {y.x, y.y, y.z, y.w};
      float e = 0.0f, l = 0.0f;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        float const err = (v[i] + s.b3[i]) - yy[i];
        e = fmaxf(e, fabsf(err));
        l += err * err;
        d[i] = 2.0f * err * inv_batch;
      }
      float const ct = expf(-AF_CONF_K * e);
      float const c = 1.0f / (1.0f + expf(-(v[4] + s.b3[4])));
      l -= ct * logf(c + 1e-12f) + (1.0f - ct) * logf(1.0f - c + 1e-12f);
      d[4] = (c - ct) * inv_batch;
      lsum += l;
    }
    put8(s.dout, tid, 0, AF_N3, d);
    put8(s.dout, tid, 8, AF_N3, d + 8);
#pragma unroll
    for (int o = 0; o < 16; ++o) put_t(s.bt1, 64 + o, tid, d[o]);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    ok = ok && layer_mma(tm + TM_DH2, s.dout, s.w3t, AF_N3, AF_H, 0, &s.bar, phase);
    float pre[16];
#pragma unroll
    for (int c = 0; c < AF_H; c += 16) {
      tmem_ld16(lane_addr(tm, TM_DH2 + c), v);
      tmem_ld16(lane_addr(tm, TM_D2 + c), pre);
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        v[i] *= gelu_grad(pre[i] + s.b2[c + i]);
        put_t(s.bt1, c + i, tid, v[i]);
      }
      put8(s.dh2, tid, c, AF_H, v);
      put8(s.dh2, tid, c + 8, AF_H, v + 8);
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    ok = ok && layer_mma(tm + TM_DH1, s.dh2, s.w2t, AF_H, AF_H, 0, &s.bar, phase);
#pragma unroll
    for (int c = 0; c < AF_H; c += 16) {
      tmem_ld16(lane_addr(tm, TM_DH1 + c), v);
      tmem_ld16(lane_addr(tm, TM_D1 + c), pre);
#pragma unroll
      for (int i = 0; i < 16; ++i) put_t(s.bt2, c + i, tid, v[i] * gelu_grad(pre[i] + s.b1[c + i]));
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    // weight and bias gradients, accumulated over the CTA's tiles
    if (tid == 0) {
      tc_fence_after();
      for (uint32_t ks = 0; ks < AF_TILE / 16; ++ks) {
        uint32_t const acc = (any || ks > 0) ? 1u : 0u;
        mma_bf16(tm + TM_G1, tile_desc(s.a1, AF_TILE, ks), tile_desc(s.bt1, AF_TILE, ks), idesc_bf16(128, 80), acc);
        mma_bf16(tm + TM_G2, tile_desc(s.a2, AF_TILE, ks), tile_desc(s.bt2, AF_TILE, ks), idesc_bf16(128, 64), acc);
        mma_bf16(tm + TM_G3, tile_desc(s.a2, AF_TILE, ks), tile_desc(s.bt1, AF_TILE, ks), idesc_bf16(128, 80), acc);
      }
      mma_commit(&s.bar);
    }
    ok = ok && mbar_wait(&s.bar, phase);
    phase ^= 1u;
    tc_fence_after();
    any = true;
  }
  // the CTA's gradients into the global accumulators
  if (any && ok) {
    float g[16];
    uint32_t const r = tid;  // tensor-memory row = transposed-operand row
#pragma unroll 1
    for (int c = 0; c < 80; c += 16) {
      tmem_ld16(lane_addr(tm, TM_G1 + c), g);
      for (int i = 0; i < 16; ++i) {
        int const o = c + i;
        if (r < 64 && o < 64) atomicAdd(&M.grads[AF_OFF_W2 + o * AF_H + r], g[i]);
        if (r >= 64 && o >= 64 && o < 64 + AF_O) atomicAdd(&M.grads[AF_OFF_W3 + (o - 64) * AF_H + (r - 64)], g[i]);
      }
    }
#pragma unroll 1
    for (int c = 0; c < 64; c += 16) {
      tmem_ld16(lane_addr(tm, TM_G2 + c), g);
      for (int i = 0; i < 16; ++i) {
        int const o = c + i;
        if (r < AF_F) atomicAdd(&M.grads[AF_OFF_W1 + o * AF_F + r], g[i]);
        if (r == AF_ONES_ROW) atomicAdd(&M.grads[AF_OFF_B1 + o], g[i]);
      }
    }
#pragma unroll 1
    for (int c = 0; c < 80; c += 16) {
      tmem_ld16(lane_addr(tm, TM_G3 + c), g);
      for (int i = 0; i < 16; ++i) {
        int const o = c + i;
        if (r == AF_ONES_ROW && o < 64) atomicAdd(&M.grads[AF_OFF_B2 + o], g[i]);
        if (r == AF_ONES_ROW && o >= 64 && o < 64 + AF_O) atomicAdd(&M.grads[AF_OFF_B3 + (o - 64)], g[i]);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xFFFFFFFFu, lsum, o);
  if ((tid & 31) == 0) atomicAdd(&s.loss, lsum);
  if (!ok && tid == 0) atomicOr(status, 1u);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (tid == 0 && loss_out) atomicAdd(loss_out, s.loss);
  if (tid < 32) tmem_dealloc(tm, 512);
}

// Adam on the fp32 masters; clears the gradient accumulators.
__global__ void k_af_adam(AfModelDev M, float lr, float beta1, float beta2, float eps, float bc1, float bc2) {
  int const i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= AF_PARAMS) return;
  float const g = M.grads[i];
  float const m = beta1 * M.adam_m[i] + (1.0f - beta1) * g;
  float const v = beta2 * M.adam_v[i] + (1.0f - beta2) * g * g;
  M.adam_m[i] = m;
  M.adam_v[i] = v;
  M.params[i] -= lr * (m / bc1) / (sqrtf(v / bc2) + eps);
  M.grads[i] = 0.0f;
}

cudaError_t launch_af_train(AfModelDev const& M, uint16_t const* X, float4 const* Y, uint32_t n, float inv_batch,
                            float* loss_out, unsigned int* status, uint32_t num_sms, cudaStream_t s) {
  uint32_t tiles = (n + AF_TILE - 1) / AF_TILE;
  uint32_t grid = tiles < num_sms ? tiles : num_sms;
  if (grid) k_af_train<<<grid, AF_TILE, sizeof(TrainSmem), s>>>(M, X, Y, n, inv_batch, loss_out, status);
  return cudaGetLastError();
}

// The training and inference kernels' shared-memory limits, set on the
// current device (function attributes are per device).
cudaError_t init_learned() {
  cudaError_t e = cudaFuncSetAttribute(k_af_train, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(sizeof(TrainSmem)));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_af_infer, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              static_cast<int>(sizeof(InferSmem)));
}

void launch_af_adam(AfModelDev const& M, float lr, uint32_t step, cudaStream_t s) {
  float const b1 = 0.9f, b2 = 0.999f;
  float const bc1 = 1.0f - powf(b1, static_cast<float>(step)), bc2 = 1.0f - powf(b2, static_cast<float>(step));
  k_af_adam<<<(AF_PARAMS + 255) / 256, 256, 0, s>>>(M, lr, b1, b2, 1e-8f, bc1, bc2);
}

void launch_af_pack(AfModelDev const& M, cudaStream_t s) { k_af_pack<<<1, 256, 0, s>>>(M); }

cudaError_t launch_af_infer(AfModelDev const& M, uint16_t const* X, float4 const* skip, uint32_t n, float* out,
                            unsigned int* status, uint32_t num_sms, cudaStream_t s) {
  uint32_t tiles = (n + AF_TILE - 1) / AF_TILE;
  uint32_t grid = tiles < num_sms ? tiles : num_sms;
  if (grid) k_af_infer<<<grid, AF_TILE, sizeof(InferSmem), s>>>(M, X, skip, n, out, status);
  return cudaGetLastError();
}

}  // namespace sg
