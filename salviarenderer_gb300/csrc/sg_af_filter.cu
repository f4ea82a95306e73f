// sg_af_filter.cu -- the learned anisotropic filter inside a pass: the
// lookups k_shade queued for SG_PS_TEX_GRAD_LEARNED draws are filtered here,
// between shading and output merging.
//
//   k_af_filter    128 lookups per tile: each thread decides whether the
//                  network applies to its lookup (a minified lookup of an
//                  anisotropic sampler with more than 4 probes -- fewer cost
//                  no more than the network's own four taps -- and at most
//                  the draw's constants[1]) and forms its 24 features (four
//                  bilinear taps along the major axis); the three layers run
//                  on tcgen05.mma with the accumulators in tensor memory, and
//                  the epilogue writes the modulated prediction into the
//                  fragment's colour -- or, for a lookup the network does not
//                  apply to or whose confidence is below the draw's
//                  constants[0], queues it for the plain sampler.
//   k_af_fallback  the plain anisotropic sampler (sampler::sample_2d_grad,
//                  sampler.cpp:854-873) for the queued lookups.
// The k_shade instances of those draws are compiled here too.
#include <cuda_runtime.h>

#include "sg_af_mma.cuh"
#include "sg_raster.cuh"

namespace sg {

struct FilterSmem {
  uint8_t w1[AF_H * AF_K1 * 2], w2[AF_H * AF_H * 2], w3[AF_N3 * AF_H * 2];
  uint8_t x[AF_TILE * AF_K1 * 2], h1[AF_TILE * AF_H * 2], h2[AF_TILE * AF_H * 2];
  float b1[AF_H], b2[AF_H], b3[AF_N3];
  uint64_t bar;
  uint32_t tmem;
};
constexpr uint32_t FILTER_CTAS_PER_SM = 4;   // 4 x 128 tensor-memory columns = all 512
constexpr uint32_t FILTER_TMEM_COLS = 128;    // layer 1 and 3 at column 0, layer 2 at 64

__device__ inline bool unorm_format(uint32_t fmt) { return fmt == SG_FMT_RGBA8 || fmt == SG_FMT_BGRA8; }

__global__ void __launch_bounds__(AF_TILE, FILTER_CTAS_PER_SM) k_af_filter(PassParams P, AfModelDev M) {
  if (P.counters->overflow & (OVF_BIN | OVF_FRAG | OVF_REC)) return;
  uint32_t const n = min(P.counters->af_lookups, P.af_capacity);
  if (blockIdx.x * AF_TILE >= n) return;  // no tile for this CTA: no tensor memory either
  extern __shared__ __align__(128) uint8_t smem_raw[];
  FilterSmem& s = *reinterpret_cast<FilterSmem*>(smem_raw);
  uint32_t const tid = threadIdx.x;
  if (tid < 32) tmem_alloc(&s.tmem, FILTER_TMEM_COLS);
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
    bool const valid = row < n;
    float f[AF_F];
    float4 r1 = make_float4(0, 0, 0, 0), mod = make_float4(0, 0, 0, 0);
    float skip[4] = {0, 0, 0, 0};
    uint32_t draw = 0;
    bool take = false;
    if (valid) {
      float4 const* L = P.af_lookups + static_cast<size_t>(row) * AF_LOOKUP_UNITS;
      float4 const r0 = L[0];
      r1 = L[1];
      mod = L[2];
      draw = __float_as_uint(r1.w);
      DrawParams const& D = P.draws[draw];
      dev_sampler const& S = D.ps_samp;
      if (S.mip_filter == SG_FILTER_ANISOTROPIC && S.max_anisotropy > 1) {
        af_info af;
        af_features(S, r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, f, af);
        take = af.lod >= 0.0f && af.probe_count > 4.0f && af.probe_count <= D.ps_k[1];
      }
    }
    if (take) {
#pragma unroll
      for (int c = 0; c < 4; ++c) skip[c] = af_skip(f, c);
    } else {
#pragma unroll
      for (int k = 0; k < AF_F; ++k) f[k] = 0.0f;
    }
    float fz[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    put8(s.x, tid, 0, AF_K1, f);
    put8(s.x, tid, 8, AF_K1, f + 8);
    put8(s.x, tid, 16, AF_K1, f + 16);
    put8(s.x, tid, 24, AF_K1, fz);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    ok = ok && layer_mma(tm, s.x, s.w1, AF_K1, AF_H, 0, &s.bar, phase);
    float v[16];
#pragma unroll
    for (int c = 0; c < AF_H; c += 16) {
      tmem_ld16(lane_addr(tm, c), v);
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] = gelu(v[i] + s.b1[c + i]);
      put8(s.h1, tid, c, AF_H, v);
      put8(s.h1, tid, c + 8, AF_H, v + 8);
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    ok = ok && layer_mma(tm + 64, s.h1, s.w2, AF_H, AF_H, 0, &s.bar, phase);
#pragma unroll
    for (int c = 0; c < AF_H; c += 16) {
      tmem_ld16(lane_addr(tm, 64 + c), v);
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] = gelu(v[i] + s.b2[c + i]);
      put8(s.h2, tid, c, AF_H, v);
      put8(s.h2, tid, c + 8, AF_H, v + 8);
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    ok = ok && layer_mma(tm, s.h2, s.w3, AF_H, AF_N3, 0, &s.bar, phase);
    tmem_ld16(lane_addr(tm, 0), v);
    bool fallback = valid && ok && !take;
    if (take && ok) {
      DrawParams const& D = P.draws[draw];
      float const conf = 1.0f / (1.0f + expf(-(v[4] + s.b3[4])));
      if (conf >= D.ps_k[0]) {
        float c[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          c[i] = skip[i] + (v[i] + s.b3[i]);
          if (unorm_format(D.ps_samp.fmt)) c[i] = fminf(fmaxf(c[i], 0.0f), 1.0f);
        }
        P.frag_color[__float_as_uint(r1.z)] = make_float4(c[0] * mod.x, c[1] * mod.y, c[2] * mod.z, c[3] * mod.w);
      } else {
        fallback = true;
      }
    }
    // queue the lookups the filter is not confident about, one atomic per warp
    unsigned const fb = __ballot_sync(0xFFFFFFFFu, fallback);
    if (fb) {
      int const lane = tid & 31, leader = __ffs(fb) - 1;
      uint32_t first = 0;
      if (lane == leader) first = atomicAdd(&P.counters->af_fallbacks, static_cast<unsigned>(__popc(fb)));
      first = __shfl_sync(0xFFFFFFFFu, first, leader);
      if (fallback) P.af_fallback[first + __popc(fb & ((1u << lane) - 1u))] = row;
    }
    tc_fence_before();
    __syncthreads();
  }
  if (!ok && tid == 0) atomicOr(&P.counters->overflow, OVF_AF_TIMEOUT);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (tid < 32) tmem_dealloc(tm, FILTER_TMEM_COLS);
}

__global__ void __launch_bounds__(256) k_af_fallback(PassParams P) {
  if (P.counters->overflow & (OVF_BIN | OVF_FRAG | OVF_REC)) return;
  uint32_t const n = P.counters->af_fallbacks;  // at most the lookups filtered, which fit the queue
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float4 const* L = P.af_lookups + static_cast<size_t>(P.af_fallback[i]) * AF_LOOKUP_UNITS;
    float4 const r0 = L[0], r1 = L[1], m = L[2];
    DrawParams const& D = P.draws[__float_as_uint(r1.w)];
    v4 const t = sample_2d_grad(D.ps_samp, r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, 0.0f);
    P.frag_color[__float_as_uint(r1.z)] = make_float4(t.x * m.x, t.y * m.y, t.z * m.z, t.w * m.w);
  }
}

void launch_af_pass(PassParams const& P, AfModelDev const& M, uint32_t num_sms, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_af_filter, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sizeof(FilterSmem)));
    attr = true;
  }
  k_af_filter<<<num_sms * FILTER_CTAS_PER_SM, AF_TILE, sizeof(FilterSmem), s>>>(P, M);
  k_af_fallback<<<num_sms * 4, 256, 0, s>>>(P);
}

// Adds the pass's learned-filter counts to the device's profile totals.
__global__ void k_af_count(PassParams P, unsigned long long* acc) {
  if (P.counters->overflow & (OVF_BIN | OVF_FRAG | OVF_REC)) return;
  acc[0] += min(P.counters->af_lookups, P.af_capacity);
  acc[1] += P.counters->af_fallbacks;
}
void launch_af_count(PassParams const& P, unsigned long long* acc, cudaStream_t s) { k_af_count<<<1, 1, 0, s>>>(P, acc); }

// k_shade for learned-filter draws (shade class 8 + na, na >= 2 varyings).
void launch_shade_learned(uint32_t na, PassParams const& P, uint32_t grid, cudaStream_t s) {
  switch (na) {
  case 2: launch_shade_learned_t<2>(P, grid, s); break;
  case 3: launch_shade_learned_t<3>(P, grid, s); break;
  case 4: launch_shade_learned_t<4>(P, grid, s); break;
  case 5: launch_shade_learned_t<5>(P, grid, s); break;
  default: break;
  }
}

// The EWA table of this translation unit's sampler.
cudaError_t upload_ewa_table_filter(float const* tab, cudaStream_t s) {
  return cudaMemcpyToSymbolAsync(c_ewa, tab, 256 * sizeof(float), 0, cudaMemcpyHostToDevice, s);
}

}  // namespace sg
