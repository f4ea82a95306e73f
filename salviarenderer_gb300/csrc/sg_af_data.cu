// sg_af_data.cu -- training samples of the learned anisotropic filter: random
// lookups on the training textures, their features and the plain
// anisotropic sampler's result (sampler::sample_2d_grad, sampler.cpp:854-873)
// as the target.
#include <cuda_runtime.h>

#include <cuda_bf16.h>

#include "sg_learned.cuh"

namespace sg {

__device__ inline uint64_t hash64(uint64_t x) {
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
__device__ inline float unit(uint64_t& st) {
  st += 0x9E3779B97F4A7C15ull;
  return static_cast<float>((hash64(st) >> 40) * (1.0 / 16777216.0));
}

// Lookup i: texture i mod ntex, uniform (u, v), a minor axis of 2^U(0, 7)
// texels and an anisotropy ratio U(2.5, 16) (the lookups the filter takes:
// minified, more than 4 probes), the major axis at a uniform angle and the
// minor one perpendicular; the two axes are ddx / ddy in random order.
// Y receives the plain sampler's result, less the filter's tap mean when
// `residual` is set (the network's training target).
__global__ void k_af_samples(dev_sampler const* samplers, uint32_t ntex, uint32_t n, uint32_t first, uint64_t seed,
                             uint16_t* X, float4* Y, float* features_f32, bool residual) {
  uint32_t const i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t st = hash64(seed * 0x100000001B3ull + first + i);
  dev_sampler const& s = samplers[(first + i) % ntex];
  float const u = unit(st), v = unit(st);
  float const minor = exp2f(7.0f * unit(st));
  float const major = minor * (2.5f + 13.5f * unit(st));
  float const ang = 3.14159265358979f * unit(st);
  float const ca = cosf(ang), sa = sinf(ang);
  float ax = major * ca, ay = major * sa, bx = -minor * sa, by = minor * ca;
  if (unit(st) < 0.5f) {
    float tx = ax, ty = ay;
    ax = bx;
    ay = by;
    bx = tx;
    by = ty;
  }
  float const fw = static_cast<float>(s.width), fh = static_cast<float>(s.height);
  float const dxu = ax / fw, dxv = ay / fh, dyu = bx / fw, dyv = by / fh;
  float f[AF_F];
  af_info af;
  af_features(s, u, v, dxu, dxv, dyu, dyv, f, af);
  v4 const t = sample_2d_grad(s, u, v, dxu, dxv, dyu, dyv, 0.0f);
  if (residual)
    Y[i] = make_float4(t.x - af_skip(f, 0), t.y - af_skip(f, 1), t.z - af_skip(f, 2), t.w - af_skip(f, 3));
  else
    Y[i] = make_float4(t.x, t.y, t.z, t.w);
  uint16_t* x = X + static_cast<size_t>(i) * AF_K1;
#pragma unroll
  for (int k = 0; k < AF_K1; ++k) x[k] = k < AF_F ? __bfloat16_as_ushort(__float2bfloat16_rn(f[k])) : 0;
  if (features_f32)
    for (int k = 0; k < AF_F; ++k) features_f32[static_cast<size_t>(i) * AF_F + k] = f[k];
}

void launch_af_samples(dev_sampler const* samplers, uint32_t ntex, uint32_t n, uint32_t first, uint64_t seed,
                       uint16_t* X, float4* Y, float* features_f32, bool residual, cudaStream_t s) {
  if (n) k_af_samples<<<(n + 127) / 128, 128, 0, s>>>(samplers, ntex, n, first, seed, X, Y, features_f32, residual);
}

// ---------------------------------------------------------------------------
// Procedural training textures (RGBA8, size x size, tileable): kind 0 value
// noise, 1 checkerboard, 2 sinusoidal grating; the parameters come from a
// hash of (seed, texture index).

__device__ inline float lattice(uint64_t key, int x, int y, int c) {
  uint64_t const h = hash64(key ^ (static_cast<uint64_t>(x) * 0x9E3779B1ull) ^ (static_cast<uint64_t>(y) << 32) ^
                            (static_cast<uint64_t>(c) << 58));
  return static_cast<float>((h >> 40) * (1.0 / 16777216.0));
}

__global__ void k_af_pattern(uint8_t* dst, uint32_t size, uint64_t seed, uint32_t index) {
  uint32_t const x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= size) return;
  uint64_t st = hash64(seed * 0x100000001B3ull + index);
  uint32_t const kind = index % 3u;
  float rgba[4];
  if (kind == 0) {  // value noise: octaves of a smoothstep-interpolated random lattice, tileable
    int const base = 2 << (hash64(st + 1) % 3);           // 2, 4 or 8 cells
    int const octaves = 4 + static_cast<int>(hash64(st + 2) % 5);
    for (int c = 0; c < 4; ++c) {
      float v = 0.0f, amp = 1.0f, sum = 0.0f;
      for (int o = 0; o < octaves; ++o) {
        int const cells = base << o;
        if (cells > static_cast<int>(size)) break;
        float const fx = (static_cast<float>(x) + 0.5f) * cells / size, fy = (static_cast<float>(y) + 0.5f) * cells / size;
        int const ix = static_cast<int>(floorf(fx)), iy = static_cast<int>(floorf(fy));
        float tx = fx - ix, ty = fy - iy;
        tx = tx * tx * (3.0f - 2.0f * tx);
        ty = ty * ty * (3.0f - 2.0f * ty);
        uint64_t const key = st * 31 + o;
        int const x0 = ix % cells, x1 = (ix + 1) % cells, y0 = iy % cells, y1 = (iy + 1) % cells;
        float const a = lattice(key, x0, y0, c), b = lattice(key, x1, y0, c);
        float const d = lattice(key, x0, y1, c), e = lattice(key, x1, y1, c);
        v += amp * ((a + (b - a) * tx) + ((d + (e - d) * tx) - (a + (b - a) * tx)) * ty);
        sum += amp;
        amp *= 0.5f;
      }
      rgba[c] = v / sum;
    }
  } else if (kind == 1) {  // checkerboard, period 2-64 texels, two random colours
    uint32_t const period = 2u << (hash64(st + 3) % 6);
    bool const odd = (((x / period) + (y / period)) & 1u) != 0u;
    for (int c = 0; c < 4; ++c) rgba[c] = lattice(st, odd ? 1 : 0, 7, c);
  } else {  // sinusoidal grating at a random orientation, period 2-64 texels, tileable
    float const ang = 6.2831853f * lattice(st, 3, 3, 0);
    float const k = static_cast<float>(size) / exp2f(1.0f + 5.0f * lattice(st, 4, 4, 0));  // cycles per texture
    float const kx = rintf(k * cosf(ang)), ky = rintf(k * sinf(ang));
    float const t = 6.2831853f * (kx * static_cast<float>(x) + ky * static_cast<float>(y)) / static_cast<float>(size);
    for (int c = 0; c < 4; ++c) rgba[c] = 0.5f + 0.5f * sinf(t + 6.2831853f * lattice(st, 5, 5, c));
  }
  uint8_t* p = dst + (static_cast<size_t>(y) * size + x) * 4;
  for (int c = 0; c < 4; ++c) p[c] = static_cast<uint8_t>(fminf(fmaxf(rintf(rgba[c] * 255.0f), 0.0f), 255.0f));
}

void launch_af_pattern(uint8_t* dst, uint32_t size, uint64_t seed, uint32_t index, cudaStream_t s) {
  k_af_pattern<<<dim3((size + 127) / 128, size), 128, 0, s>>>(dst, size, seed, index);
}

// The EWA table of this translation unit's sampler.
cudaError_t upload_ewa_table_af(float const* tab, cudaStream_t s) {
  return cudaMemcpyToSymbolAsync(c_ewa, tab, 256 * sizeof(float), 0, cudaMemcpyHostToDevice, s);
}

}  // namespace sg
