// sg_af_filter.cu -- the learned anisotropic filter inside a pass, between
// shading and output merging.  k_shade's learned instances (compiled here)
// queue each lookup of an SG_PS_TEX_GRAD_LEARNED draw either for the network
// -- with its 24 features already formed, the four taps filtered by the
// texture units -- or for the plain sampler.
//
//   k_af_filter    128 queued lookups per tile: the feature rows go to shared
//                  memory, the three layers run on tcgen05.mma with the
//                  accumulators in tensor memory, and the epilogue writes the
//                  modulated prediction (tap mean + network) into the
//                  fragment's colour -- or, below the draw's confidence
//                  threshold (constants[0]), queues the lookup for the plain
//                  sampler.
//   k_af_fallback  the plain anisotropic sampler (sampler::sample_2d_grad,
//                  sampler.cpp:854-873) for the network's rejects and for the
//                  lookups k_shade queued for it.
#include <cuda_runtime.h>

#include "sg_af_mma.cuh"
#include "sg_raster.cuh"

namespace sg {

// One activation tile serves both hidden layers: layer 2's MMA has read h1
// by the time its epilogue writes h2 over it.  `rec` receives a tile's
// queue records by one bulk copy, issued for the next tile as soon as the
// threads have taken the current one out.
struct FilterSmem {
  float4 rec[AF_TILE * AF_NET_UNITS];
  uint8_t w1[AF_H * AF_K1 * 2], w2[AF_H * AF_H * 2], w3[AF_N3 * AF_H * 2];
  uint8_t x[AF_TILE * AF_K1 * 2], h[AF_TILE * AF_H * 2];
  float b1[AF_H], b2[AF_H], b3[AF_N3];
  uint64_t bar, lbar;
  uint32_t tmem;
};
constexpr uint32_t FILTER_CTAS_PER_SM = 4;  // 55 KB of shared memory each
// Every layer's accumulator at column 0: each epilogue has read the previous
// one (tcgen05.wait::ld) before the barrier that precedes the next MMA.
constexpr uint32_t FILTER_TMEM_COLS = 64;

__device__ inline bool unorm_format(uint32_t fmt) { return fmt == SG_FMT_RGBA8 || fmt == SG_FMT_BGRA8; }

__global__ void __launch_bounds__(AF_TILE, FILTER_CTAS_PER_SM) k_af_filter(PassParams P, AfModelDev M) {
  pdl_wait();
  if ((P.counters->overflow & OVF_FATAL) || pass_gated(P)) return;
  uint32_t const n = min(P.counters->af_lookups, P.af_net_capacity);
  if (blockIdx.x * AF_TILE >= n) return;  // no tile for this CTA: no tensor memory either
  extern __shared__ __align__(128) uint8_t smem_raw[];
  FilterSmem& s = *reinterpret_cast<FilterSmem*>(smem_raw);
  uint32_t const tid = threadIdx.x;
  uint32_t const stride = gridDim.x * AF_TILE;
  // thread 0: the records of the tile at `t` into s.rec
  auto issue = [&](uint32_t t) {
    uint32_t const bytes = min(static_cast<uint32_t>(AF_TILE), n - t) * AF_NET_UNITS * static_cast<uint32_t>(sizeof(float4));
    mbar_expect_tx(&s.lbar, bytes);
    bulk_g2s(s.rec, P.af_net + static_cast<size_t>(t) * AF_NET_UNITS, bytes, &s.lbar);
  };
  if (tid < 32) tmem_alloc(&s.tmem, FILTER_TMEM_COLS);
  if (tid == 0) {
    mbar_init(&s.bar, 1);
    mbar_init(&s.lbar, 1);
    issue(blockIdx.x * AF_TILE);
  }
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
  uint32_t phase = 0, lphase = 0;
  bool ok = true, inflight = true;  // inflight: a bulk copy into s.rec not yet waited for
  for (uint32_t t0 = blockIdx.x * AF_TILE; t0 < n && ok; t0 += stride) {
    uint32_t const row = t0 + tid;
    bool const valid = row < n;
    if (__syncthreads_or(!mbar_wait(&s.lbar, lphase))) {  // the CTA leaves together
      ok = false;
      break;
    }
    lphase ^= 1u;
    inflight = false;
    // this row's record: the feature row into the A tile, the tap mean,
    // pixel and draw, and modulation into registers (units read in an order
    // rotated by row, so that the threads of a warp hit distinct banks)
    float4 skip = make_float4(0, 0, 0, 0), r1 = skip, mod = skip;
#pragma unroll
    for (uint32_t j = 0; j < AF_NET_UNITS; ++j) {
      uint32_t const u = (j + tid) & (AF_NET_UNITS - 1);
      if (u == 5) continue;  // the plain sampler's coordinates: for the fallback only
      float4 const v = valid ? s.rec[tid * AF_NET_UNITS + u] : make_float4(0, 0, 0, 0);
      if (u < AF_K1 / 8)
        *reinterpret_cast<float4*>(s.x + tile_off(tid, 8 * u, AF_K1)) = v;
      else if (u == 4)
        skip = v;
      else if (u == 6)
        r1 = v;
      else
        mod = v;
    }
    __syncthreads();  // s.rec is free: the next tile's records come in during this tile's layers
    if (t0 + stride < n) {
      if (tid == 0) {
        fence_async_smem();
        issue(t0 + stride);
      }
      inflight = true;
    }
    // the draw's confidence threshold and texel format, read before the layers
    float thr = 0.0f;
    bool unorm = false;
    if (valid) {
      DrawParams const& D = P.draws[__float_as_uint(r1.w)];
      thr = D.ps_k[0];
      unorm = unorm_format(D.ps_samp.fmt);
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    ok = ok && layer_mma(tm, s.x, s.w1, AF_K1, AF_H, 0, &s.bar, phase);
    float v[16];
#pragma unroll
    for (int c = 0; c < AF_H; c += 16) {
      tmem_ld16(lane_addr(tm, c), v);
      gelu_row16(s.h, tid, c, AF_H, v, s.b1 + c);
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    ok = ok && layer_mma(tm, s.h, s.w2, AF_H, AF_H, 0, &s.bar, phase);
#pragma unroll
    for (int c = 0; c < AF_H; c += 16) {
      tmem_ld16(lane_addr(tm, c), v);
      gelu_row16(s.h, tid, c, AF_H, v, s.b2 + c);
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    ok = ok && layer_mma(tm, s.h, s.w3, AF_H, AF_N3, 0, &s.bar, phase);
    tmem_ld16(lane_addr(tm, 0), v);
    bool fallback = false;
    if (valid && ok) {
      float const conf = 1.0f / (1.0f + expf(-(v[4] + s.b3[4])));
      if (conf >= thr) {
        float c[4];
        float const k4[4] = {skip.x, skip.y, skip.z, skip.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          c[i] = k4[i] + (v[i] + s.b3[i]);
          if (unorm) c[i] = fminf(fmaxf(c[i], 0.0f), 1.0f);
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
  // a copy still in flight (after a timeout) lands before the CTA ends
  if (inflight) mbar_wait(&s.lbar, lphase);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (tid < 32) tmem_dealloc(tm, FILTER_TMEM_COLS);
}

__global__ void __launch_bounds__(256) k_af_fallback(PassParams P) {
  pdl_wait();
  if ((P.counters->overflow & OVF_FATAL) || pass_gated(P)) return;
  // the network's rejects (af_fallback into af_net), then the lookups
  // k_shade queued for the plain sampler (af_plain)
  uint32_t const nf = P.counters->af_fallbacks;
  uint32_t const n = nf + min(P.counters->af_plain, P.af_capacity);  // (all of them: else OVF_AF_QUEUE)
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float4 const* L = i < nf ? P.af_net + static_cast<size_t>(P.af_fallback[i]) * AF_NET_UNITS + 5
                             : P.af_plain + static_cast<size_t>(i - nf) * AF_PLAIN_UNITS;
    float4 const r0 = L[0], r1 = L[1], m = L[2];
    DrawParams const& D = P.draws[__float_as_uint(r1.w)];
    v4 const t = sample_2d_grad(D.ps_samp, r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, 0.0f);
    P.frag_color[__float_as_uint(r1.z)] = make_float4(t.x * m.x, t.y * m.y, t.z * m.z, t.w * m.w);
  }
}

void launch_af_pass(PassParams const& P, AfModelDev const& M, uint32_t num_sms, cudaStream_t s) {
  launch_pdl(k_af_filter, num_sms * FILTER_CTAS_PER_SM, AF_TILE, sizeof(FilterSmem), s, P, M);
  launch_pdl(k_af_fallback, num_sms * 4, 256, 0, s, P);
}

// k_af_filter's shared-memory limit on the current device.
cudaError_t init_af_filter() {
  return cudaFuncSetAttribute(k_af_filter, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              static_cast<int>(sizeof(FilterSmem)));
}

// Adds the pass's learned-filter counts to the device's profile totals.
__global__ void k_af_count(PassParams P, unsigned long long* acc) {
  if ((P.counters->overflow & OVF_FATAL) || pass_gated(P)) return;
  acc[0] += min(P.counters->af_lookups, P.af_net_capacity);
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
