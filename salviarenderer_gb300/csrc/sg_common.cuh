// sg_common.cuh -- device numerics, pixel formats and the software sampler.
//
// Every function reproduces the float semantics of the reference CPU
// renderer operation by operation (the file compiles with -fmad=false, so
// no multiply-add is contracted; divisions and square roots are IEEE
// round-to-nearest).  Reference lines are cited per function.
#pragma once

#include <cuda_fp16.h>

#include <cstdint>

#include "salvia_gb300.h"

namespace sg {

// ---------------------------------------------------------------------------
// eflib numerics (eflib/include/eflib/math/math.h:21-164)
__host__ __device__ inline float smin(float a, float b) { return (b < a) ? b : a; }  // std::min
__host__ __device__ inline float smax(float a, float b) { return (a < b) ? b : a; }  // std::max
__host__ __device__ inline float sse_min(float a, float b) { return a < b ? a : b; }  // _mm_min_ps
__host__ __device__ inline float sse_max(float a, float b) { return a > b ? a : b; }  // _mm_max_ps
__host__ __device__ inline float sclamp(float v, float lo, float hi) {             // std::clamp
  return (v < lo) ? lo : ((hi < v) ? hi : v);
}
__host__ __device__ inline int iclamp(int v, int lo, int hi) { return (v < lo) ? lo : ((hi < v) ? hi : v); }

__device__ inline bool eq_eps(float a, float b) {  // equal<float> (math.h:21-26)
  return fabsf(a - b) <= 1.1920928955078125e-07f;
}
__device__ inline float fast_round(float val) {  // math.h:112-126
  uint32_t n = __float_as_uint(val);
  float bias = __uint_as_float(((23u + 127u) << 23) + (n & 0x80000000u));
  float f = __fadd_rn(val, bias);
  return __fsub_rn(f, bias);
}
__device__ inline float fast_floor(float val) {  // math.h:133-136
  float f = fast_round(val);
  return (f > val) ? f - 1.0f : f;
}
// fast_roundi / fast_floori / fast_ceili take a double (math.h:139-164):
// floor(d + 0.5) with the 0.5 - 1.5e-8 bias of the floori/ceili forms,
// evaluated in double exactly as the reference does.
__device__ inline int fast_roundi(double d) { return static_cast<int>(floor(d + 0.5)); }
#define SG_ROUND_EPS (static_cast<double>(0.5f) - 1.5e-8)
__device__ inline int fast_floori(double d) { return fast_roundi(d - SG_ROUND_EPS); }
__device__ inline int fast_ceili(double d) { return fast_roundi(d + SG_ROUND_EPS); }
// The same three of a float argument (the reference widens it to double)
// without FP64 arithmetic, which is slow on this part.  Equal as values for
// every float (all 2^32 checked against the double forms):
// floor(double(f) + 0.5) is floor of f + 0.5 rounded down in float; the
// floori form is floor(f) except on [-0x1.01b2b2p-26, 0), where the bias
// lifts it to 0; the ceili form is ceil(f) except on (0, 0x1.01b2b2p-26],
// where it drops to 0, for |f| < 2^26 -- above that the double sum rounds
// the bias and the double form is kept.
__device__ inline int fast_roundi_f(float f) { return static_cast<int>(floorf(__fadd_rd(f, 0.5f))); }
__device__ inline int fast_floori_f(float f) {
  return (f < 0.0f && f >= -0x1.01b2b2p-26f) ? 0 : static_cast<int>(floorf(f));
}
__device__ inline int fast_ceili_f(float f) {
  if (!(fabsf(f) < 0x1p26f)) return fast_ceili(static_cast<double>(f));
  return (f > 0.0f && f <= 0x1.01b2b2p-26f) ? 0 : static_cast<int>(ceilf(f));
}
__device__ inline float fast_log2(float val) {  // math.h:89-105
  int32_t x = __float_as_int(val);
  int log_2 = ((x >> 23) & 255) - 128;
  x &= ~(255 << 23);
  x += 127 << 23;
  float f = __int_as_float(x);
  f = ((-1.0f / 3) * f + 2) * f - 2.0f / 3;
  return f + static_cast<float>(log_2);
}
// _mm_cvttps_epi32 / _mm_cvtps_epi32: out-of-range and NaN give 0x80000000
__device__ inline int32_t cvtt(float f) {
  if (!(f > -2147483904.0f && f < 2147483648.0f)) return INT32_MIN;
  return __float2int_rz(f);
}
__device__ inline int32_t cvt_rne(float f) {
  if (!(f > -2147483904.0f && f < 2147483648.0f)) return INT32_MIN;
  return __float2int_rn(f);
}
// vector_::length: sqrt in double of the float sum of squares
// (vector_generic.h:118-126).  The double square root rounded to float is
// the correctly rounded float square root (53 >= 2 * 24 + 2 bits: rounding
// twice is innocuous for sqrt; all 2^31 non-negative floats checked), so
// the float one is taken.
__device__ inline float len_sqrt(float t) { return __fsqrt_rn(t); }
__device__ inline float len2(float x, float y) {
  float t = 0.0f;
  t += x * x;
  t += y * y;
  return len_sqrt(t);
}

struct v4 {
  float x, y, z, w;
};
__device__ inline v4 mk4(float a, float b, float c, float d) { return v4{a, b, c, d}; }
__device__ inline v4 operator+(v4 a, v4 b) { return mk4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ inline v4 operator-(v4 a, v4 b) { return mk4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
__device__ inline v4 operator*(v4 a, float s) { return mk4(a.x * s, a.y * s, a.z * s, a.w * s); }
__device__ inline v4 mulv(v4 a, v4 b) { return mk4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
__device__ inline v4 ld4(float4 const* p) {
  float4 f = *p;
  return mk4(f.x, f.y, f.z, f.w);
}
__device__ inline void st4(float4* p, v4 v) { *p = make_float4(v.x, v.y, v.z, v.w); }
__device__ inline float comp(v4 const& v, int i) { return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w; }

// ---------------------------------------------------------------------------
// pixel formats (salvia/include/salvia/common/colors.h:148-458)
__host__ __device__ inline uint32_t fmt_bytes(uint32_t fmt) {
  switch (fmt) {
  case SG_FMT_RGBA32F: return 16;
  case SG_FMT_RGB32F: return 12;
  case SG_FMT_RG32F:
  case SG_FMT_RGBA16F: return 8;
  case SG_FMT_BGRA8:
  case SG_FMT_RGBA8:
  case SG_FMT_R32F:
  case SG_FMT_R32I:
  case SG_FMT_D32F:
  case SG_FMT_D24S8: return 4;
  default: return 0;
  }
}

// Byte `sel & 3` of u as a float, exactly: the byte in the low mantissa bits
// of 2^23 (one byte permute), minus 2^23 -- a byte permute and an add in
// place of an integer-to-float conversion.  `sel` is 0x7440 + the byte.
__device__ __forceinline__ float byte_to_f(uint32_t u, uint32_t sel) {
  return __uint_as_float(__byte_perm(u, 0x4B000000u, sel)) - 8388608.0f;
}
__device__ inline v4 unorm8_to_f(uint32_t r, uint32_t g, uint32_t b, uint32_t a) {  // colors.h:176-179
  const float inv_255 = 1.0f / 255;
  return mk4(static_cast<float>(r) * inv_255, static_cast<float>(g) * inv_255,
             static_cast<float>(b) * inv_255, static_cast<float>(a) * inv_255);
}
// the four bytes of an RGBA8 (rgba) or BGRA8 texel word as colors.h:176-179
// converts them
__device__ __forceinline__ v4 unorm8_word_to_f(uint32_t u, bool rgba) {
  const float inv_255 = 1.0f / 255;
  float const b0 = byte_to_f(u, 0x7440u), b1 = byte_to_f(u, 0x7441u), b2 = byte_to_f(u, 0x7442u),
              b3 = byte_to_f(u, 0x7443u);
  return rgba ? mk4(b0 * inv_255, b1 * inv_255, b2 * inv_255, b3 * inv_255)
              : mk4(b2 * inv_255, b1 * inv_255, b0 * inv_255, b3 * inv_255);
}
__device__ inline uint32_t f_to_unorm8(float c) {  // color_rgba8::assign, SSE path (colors.h:182-192)
  float m = c * 255.0f;
  m = sse_max(m, 0.0f);
  m = sse_min(m, 255.0f);
  // m is in [0, 255] (NaN became 0): adding 2^23 rounds it to the nearest
  // integer, ties to even, in the low mantissa bits -- cvt_rne's value
  return __float_as_uint(m + 8388608.0f) & 0xFFu;
}
// EXTENSION (RGBA16F): IEEE binary16, round to nearest even.
__device__ inline uint16_t f32_to_f16(float f) { return __half_as_ushort(__float2half_rn(f)); }
__device__ inline float f16_to_f32(uint16_t h) { return __half2float(__ushort_as_half(h)); }

__device__ inline v4 read_texel(uint32_t fmt, uint8_t const* p) {
  switch (fmt) {
  case SG_FMT_RGBA32F: {
    float4 f = *reinterpret_cast<float4 const*>(p);
    return mk4(f.x, f.y, f.z, f.w);
  }
  case SG_FMT_RGB32F: {
    float const* f = reinterpret_cast<float const*>(p);
    return mk4(f[0], f[1], f[2], 1.0f);
  }
  case SG_FMT_BGRA8: return unorm8_word_to_f(*reinterpret_cast<uint32_t const*>(p), false);
  case SG_FMT_RGBA8: return unorm8_word_to_f(*reinterpret_cast<uint32_t const*>(p), true);
  case SG_FMT_R32F: return mk4(*reinterpret_cast<float const*>(p), 0.0f, 0.0f, 0.0f);
  case SG_FMT_RG32F: {
    float2 f = *reinterpret_cast<float2 const*>(p);
    return mk4(f.x, f.y, 0.0f, 0.0f);
  }
  case SG_FMT_R32I: return mk4(static_cast<float>(*reinterpret_cast<int32_t const*>(p)), 0.0f, 0.0f, 0.0f);
  case SG_FMT_RGBA16F: {
    uint2 u = *reinterpret_cast<uint2 const*>(p);
    return mk4(f16_to_f32(u.x & 0xFFFF), f16_to_f32(u.x >> 16), f16_to_f32(u.y & 0xFFFF),
               f16_to_f32(u.y >> 16));
  }
  default: return mk4(0, 0, 0, 0);
  }
}

__device__ inline void write_texel(uint32_t fmt, uint8_t* p, v4 c) {
  switch (fmt) {
  case SG_FMT_RGBA32F: *reinterpret_cast<float4*>(p) = make_float4(c.x, c.y, c.z, c.w); break;
  case SG_FMT_RGB32F: {
    float* f = reinterpret_cast<float*>(p);
    f[0] = c.x;
    f[1] = c.y;
    f[2] = c.z;
    break;
  }
  case SG_FMT_BGRA8:
    *reinterpret_cast<uint32_t*>(p) = f_to_unorm8(c.z) | (f_to_unorm8(c.y) << 8) |
                                      (f_to_unorm8(c.x) << 16) | (f_to_unorm8(c.w) << 24);
    break;
  case SG_FMT_RGBA8:
    *reinterpret_cast<uint32_t*>(p) = f_to_unorm8(c.x) | (f_to_unorm8(c.y) << 8) |
                                      (f_to_unorm8(c.z) << 16) | (f_to_unorm8(c.w) << 24);
    break;
  case SG_FMT_R32F: *reinterpret_cast<float*>(p) = c.x; break;
  case SG_FMT_RG32F: *reinterpret_cast<float2*>(p) = make_float2(c.x, c.y); break;
  case SG_FMT_R32I: *reinterpret_cast<int32_t*>(p) = static_cast<int32_t>(c.x + 0.5f); break;
  case SG_FMT_RGBA16F: {
    uint2 u;
    u.x = uint32_t(f32_to_f16(c.x)) | (uint32_t(f32_to_f16(c.y)) << 16);
    u.y = uint32_t(f32_to_f16(c.z)) | (uint32_t(f32_to_f16(c.w)) << 16);
    *reinterpret_cast<uint2*>(p) = u;
    break;
  }
  default: break;
  }
}

__device__ inline float lerp1(float a, float b, float t) { return a + (b - a) * t; }
__device__ inline v4 lerp4(v4 c0, v4 c1, v4 c2, v4 c3, float tx, float ty) {
  float r[4];
  float const* a = &c0.x;
  float const* b = &c1.x;
  float const* c = &c2.x;
  float const* d = &c3.x;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    float c01 = lerp1(a[i], b[i], tx);
    float c23 = lerp1(c[i], d[i], tx);
    r[i] = lerp1(c01, c23, ty);
  }
  return mk4(r[0], r[1], r[2], r[3]);
}

// lerp_2d of 8-bit RGBA / BGRA texels (colors.h:340-489)
__device__ inline v4 lerp_2d_unorm8(bool rgba, uint8_t const* a, uint8_t const* b, uint8_t const* c,
                                    uint8_t const* d, float tx, float ty) {
  auto ld = [&](uint8_t const* p) {
    uint32_t u = *reinterpret_cast<uint32_t const*>(p);
    float x = byte_to_f(u, 0x7440u), y = byte_to_f(u, 0x7441u), z = byte_to_f(u, 0x7442u), w = byte_to_f(u, 0x7443u);
    return rgba ? mk4(x, y, z, w) : mk4(z, y, x, w);
  };
  v4 r = lerp4(ld(a), ld(b), ld(c), ld(d), tx, ty);
  return r * (1.0f / 255);
}

// lerp_2d per format (colors.h:340-489)
__device__ inline v4 lerp_2d(uint32_t fmt, uint8_t const* a, uint8_t const* b, uint8_t const* c,
                             uint8_t const* d, float tx, float ty) {
  switch (fmt) {
  case SG_FMT_RGBA8:
  case SG_FMT_BGRA8: return lerp_2d_unorm8(fmt == SG_FMT_RGBA8, a, b, c, d, tx, ty);
  case SG_FMT_RGB32F: {
    v4 c0 = read_texel(fmt, a), c1 = read_texel(fmt, b), c2 = read_texel(fmt, c),
       c3 = read_texel(fmt, d);
    float r01 = c0.x + (c1.x - c0.x) * tx, g01 = c0.x + (c1.y - c0.y) * tx,
          b01 = c0.x + (c1.z - c0.z) * tx;
    float r23 = c2.x + (c3.x - c2.x) * tx, g23 = c2.x + (c3.y - c2.y) * tx,
          b23 = c2.x + (c3.z - c2.z) * tx;
    return mk4(r01 + (r23 - r01) * ty, r01 + (g23 - g01) * ty, r01 + (b23 - b01) * ty, 1.0f);
  }
  case SG_FMT_RG32F: {
    v4 c0 = read_texel(fmt, a), c1 = read_texel(fmt, b), c2 = read_texel(fmt, c),
       c3 = read_texel(fmt, d);
    float r01 = c0.x + (c1.x - c0.x) * tx, g01 = c0.x + (c1.y - c0.y) * tx;
    float r23 = c2.x + (c3.x - c2.x) * tx, g23 = c2.x + (c3.y - c2.y) * tx;
    return mk4(r01 + (r23 - r01) * ty, r01 + (g23 - g01) * ty, 0.0f, 0.0f);
  }
  case SG_FMT_R32F:
  case SG_FMT_R32I: {
    float c0 = read_texel(fmt, a).x, c1 = read_texel(fmt, b).x, c2 = read_texel(fmt, c).x,
          c3 = read_texel(fmt, d).x;
    float r01 = c0 + (c1 - c0) * tx;
    float r23 = c2 + (c3 - c2) * tx;
    return mk4(r01 + (r23 - r01) * ty, 0.0f, 0.0f, 0.0f);
  }
  default:
    return lerp4(read_texel(fmt, a), read_texel(fmt, b), read_texel(fmt, c), read_texel(fmt, d), tx, ty);
  }
}

// ---------------------------------------------------------------------------
// sampler (salvia/src/resource/sampler.cpp)
constexpr int SG_MAX_LEVELS = 14;

struct dev_level {
  uint8_t const* data;
  int w, h;
};

struct dev_sampler {
  uint32_t min_filter, mag_filter, mip_filter, mip_quality;
  uint32_t address_u, address_v;
  uint32_t max_anisotropy;
  uint32_t fmt;
  uint32_t esz;
  int nlevels;
  float border[4];
  uint32_t width, height;  // texture size (level 0)
  uint32_t cube;           // a cube texture: lv[0..5] are its faces, level 0 only
  dev_level lv[SG_MAX_LEVELS];
  // texture-unit copies of the levels (bilinear, the sampler's addressing),
  // for the learned filter's feature taps; 0 where the format has none
  unsigned long long af_tex[SG_MAX_LEVELS];
};

// EWA weight table (sampler.cpp:636-678), uploaded at device creation by the
// translation unit that launches the sampling kernels.
static __constant__ float c_ewa[256];

// addressers, SSE paths (sampler.cpp:19-393)
// a / fs for a texture size fs (a positive integer below 2^24): by a power
// of two the quotient is exact either way, so it is the product with the
// reciprocal (an exponent change) -- the same float without a division.
__device__ inline float div_by_size(float a, float fs) {
  uint32_t const b = __float_as_uint(fs);
  if ((b & 0x7FFFFFu) == 0u) return a * __uint_as_float(0x7F000000u - b);
  return a / fs;
}
__device__ inline void wrap_linear(float coord, int size, int& lo, int& hi, float& frac) {
  float c0 = coord - static_cast<float>(cvtt(coord));
  float fs = static_cast<float>(size);
  c0 = fs * c0;
  c0 = c0 - 0.5f;
  float ip = static_cast<float>(cvtt(c0));
  if (ip > c0) ip = ip - 1.0f;
  frac = c0 - ip;
  float big = fs * 8192.0f;
  float a0 = (ip + 0.0f) + big, a1 = (ip + 1.0f) + big;
  float d0 = static_cast<float>(cvtt(div_by_size(a0, fs))), d1 = static_cast<float>(cvtt(div_by_size(a1, fs)));
  lo = cvtt(a0 - d0 * fs);
  hi = cvtt(a1 - d1 * fs);
}
__device__ inline void mirror_linear(float coord, int size, int& lo, int& hi, float& frac) {
  int sel = fast_floori_f(coord);
  float o = ((sel & 1) ? static_cast<float>(1 + sel) - coord : coord - static_cast<float>(sel)) *
                static_cast<float>(size) - 0.5f;
  float ip = static_cast<float>(cvtt(o));
  if (ip > o) ip = ip - 1.0f;
  frac = o - ip;
  float fs = static_cast<float>(size) - 1.0f;
  lo = cvtt(sse_min(sse_max(ip + 0.0f, 0.0f), fs));
  hi = cvtt(sse_min(sse_max(ip + 1.0f, 0.0f), fs));
}
__device__ inline void clamp_linear(float coord, int size, int& lo, int& hi, float& frac) {
  float fs = static_cast<float>(size);
  float c0 = coord * fs;
  c0 = sse_max(c0, 0.5f);
  c0 = sse_min(c0, fs - 0.5f);
  c0 = c0 - 0.5f;
  float ip = static_cast<float>(cvtt(c0));
  if (ip > c0) ip = ip - 1.0f;
  frac = c0 - ip;
  float fs1 = fs - 1.0f;
  lo = cvtt(sse_min(sse_max(ip + 0.0f, 0.0f), fs1));
  hi = cvtt(sse_min(sse_max(ip + 1.0f, 0.0f), fs1));
}
__device__ inline void border_linear(float coord, int size, int& lo, int& hi, float& frac) {
  float fs = static_cast<float>(size);
  float t = coord * fs;
  t = sse_max(t, -0.5f);
  t = sse_min(t, fs - -0.5f);
  float c0 = t + -0.5f;
  float ip = static_cast<float>(cvtt(c0));
  if (ip > c0) ip = ip - 1.0f;
  frac = c0 - ip;
  int ci = cvtt(ip);
  lo = ci >= size ? -1 : ci;
  hi = ci + 1 >= size ? -1 : ci + 1;
}
__device__ inline int wrap_point(float coord, int size) {
  float c = coord - static_cast<float>(cvtt(coord));
  float fs = static_cast<float>(size);
  c = fs * c;
  float ip = static_cast<float>(cvtt(c));
  if (ip > c) ip = ip - 1.0f;
  float a = ip + fs * 8192.0f;
  float dv = static_cast<float>(cvtt(div_by_size(a, fs)));
  return cvtt(a - dv * fs);
}
__device__ inline int mirror_point(float coord, int size) {
  int sel = fast_floori_f(coord);
  float o = ((sel & 1) ? static_cast<float>(1 + sel) - coord : coord - static_cast<float>(sel)) *
            static_cast<float>(size);
  float ip = static_cast<float>(cvtt(o));
  if (ip > o) ip = ip - 1.0f;
  return cvtt(sse_min(sse_max(ip, 0.0f), static_cast<float>(size) - 1.0f));
}
__device__ inline int clamp_point(float coord, int size) {
  float fs = static_cast<float>(size);
  float c = coord * fs;
  c = sse_max(c, 0.5f);
  c = sse_min(c, fs - 0.5f);
  float ip = static_cast<float>(cvtt(c));
  if (ip > c) ip = ip - 1.0f;
  return cvtt(sse_min(sse_max(ip, 0.0f), fs - 1.0f));
}
__device__ inline int border_point(float coord, int size) {
  float fs = static_cast<float>(size);
  float t = sse_max(coord * fs, -0.5f);
  float c = sse_min(t, fs - -0.5f);
  float ip = static_cast<float>(cvtt(c));
  if (ip > c) ip = ip - 1.0f;
  int ci = cvtt(ip);
  return ci >= size ? -1 : ci;
}
// scalar addressers for differing u/v modes (sampler.cpp:21-25,124-130,221-225,315-319,396-410)
__device__ inline float coordf(uint32_t mode, float coord, int size) {
  float fs = static_cast<float>(size);
  switch (mode) {
  case SG_ADDRESS_WRAP: return (coord - fast_floor(coord)) * fs - 0.5f;
  case SG_ADDRESS_MIRROR: {
    int sel = fast_floori_f(coord);
    return ((sel & 1) ? static_cast<float>(1 + sel) - coord : coord - static_cast<float>(sel)) * fs - 0.5f;
  }
  case SG_ADDRESS_CLAMP: return sclamp(coord * fs, 0.5f, fs - 0.5f) - 0.5f;
  default: return sclamp(coord * fs, -0.5f, fs + 0.5f) - 0.5f;
  }
}
__device__ inline int coordi_1d(uint32_t mode, int coord, int size) {
  switch (mode) {
  case SG_ADDRESS_WRAP: return (size * 8192 + coord) % size;
  case SG_ADDRESS_MIRROR:
  case SG_ADDRESS_CLAMP: return iclamp(coord, 0, size - 1);
  default: return coord >= size ? -1 : coord;
  }
}

__device__ inline v4 border_color(dev_sampler const& s) {
  return mk4(s.border[0], s.border[1], s.border[2], s.border[3]);
}

// surface_sampler::point / linear (sampler.cpp:423-483)
static __device__ __noinline__ v4 sample_surface(dev_sampler const& s, int level, float x, float y, uint32_t filter) {
  dev_level const lv = s.lv[level];
  int w = lv.w, h = lv.h;
  uint32_t mu = s.address_u, mv = s.address_v;
  auto texel = [&](int xx, int yy) -> uint8_t const* {
    return lv.data + (static_cast<size_t>(yy) * w + xx) * s.esz;
  };
  if (filter == SG_FILTER_POINT) {
    int ix, iy;
    if (mu == mv) {
      switch (mu) {
      case SG_ADDRESS_WRAP: ix = wrap_point(x, w); iy = wrap_point(y, h); break;
      case SG_ADDRESS_MIRROR: ix = mirror_point(x, w); iy = mirror_point(y, h); break;
      case SG_ADDRESS_CLAMP: ix = clamp_point(x, w); iy = clamp_point(y, h); break;
      default: ix = border_point(x, w); iy = border_point(y, h); break;
      }
      if (0 <= ix && ix < w && 0 <= iy && iy < h) return read_texel(s.fmt, texel(ix, iy));
      return border_color(s);
    }
    ix = coordi_1d(mu, fast_floori_f(coordf(mu, x, w) + 0.5f), w);
    iy = coordi_1d(mv, fast_floori_f(coordf(mv, y, h) + 0.5f), h);
    if (ix < 0 || iy < 0 || ix >= w || iy >= h) return border_color(s);
    return read_texel(s.fmt, texel(ix, iy));
  }
  int x0, x1, y0, y1;
  float tx, ty;
  if (mu == mv) {
    switch (mu) {
    case SG_ADDRESS_WRAP: wrap_linear(x, w, x0, x1, tx); wrap_linear(y, h, y0, y1, ty); break;
    case SG_ADDRESS_MIRROR: mirror_linear(x, w, x0, x1, tx); mirror_linear(y, h, y0, y1, ty); break;
    case SG_ADDRESS_CLAMP: clamp_linear(x, w, x0, x1, tx); clamp_linear(y, h, y0, y1, ty); break;
    default: border_linear(x, w, x0, x1, tx); border_linear(y, h, y0, y1, ty); break;
    }
  } else {
    float ox = coordf(mu, x, w);
    int ixp = fast_floori_f(ox);
    x0 = coordi_1d(mu, ixp, w);
    x1 = coordi_1d(mu, ixp + 1, w);
    tx = ox - static_cast<float>(ixp);
    float oy = coordf(mv, y, h);
    int iyp = fast_floori_f(oy);
    y0 = coordi_1d(mv, iyp, h);
    y1 = coordi_1d(mv, iyp + 1, h);
    ty = oy - static_cast<float>(iyp);
  }
  bool ok = x0 >= 0 && x1 >= 0 && y0 >= 0 && y1 >= 0 && x0 < w && x1 < w && y0 < h && y1 < h;
  if (ok) return lerp_2d(s.fmt, texel(x0, y0), texel(x1, y0), texel(x0, y1), texel(x1, y1), tx, ty);
  // Border addressing outside the surface: the reference forms an address
  // outside the texel array here; the border colour's storage is used instead.
  alignas(16) uint8_t tmp[16];
  write_texel(s.fmt, tmp, border_color(s));
  auto pick = [&](int xx, int yy) -> uint8_t const* {
    return (xx >= 0 && yy >= 0 && xx < w && yy < h) ? texel(xx, yy) : tmp;
  };
  return lerp_2d(s.fmt, pick(x0, y0), pick(x1, y0), pick(x0, y1), pick(x1, y1), tx, ty);
}

struct af_info {
  float lod, probe_count, weight_D, du, dv;
};

// sampler::calc_lod (sampler.cpp:521-603)
__device__ inline float calc_lod(dev_sampler const& s, float dxu, float dxv, float dyu, float dyv, float bias) {
  float sw = static_cast<float>(s.width), sh = static_cast<float>(s.height);
  if (s.mip_quality == SG_MIP_LO_QUALITY) {
    float m0 = smax(fabsf(dxu), fabsf(dyu)) * sw;
    float m1 = smax(fabsf(dxv), fabsf(dyv)) * sh;
    float m2 = smax(0.0f, 0.0f) * 1.0f;
    float rho = smax(smax(m0, m1), m2);
    return fast_log2(rho) + bias;
  }
  float dxt0 = dxu * sw, dxt1 = dxv * sh, dyt0 = dyu * sw, dyt1 = dyv * sh;
  float rho;
  if (s.mip_quality == SG_MIP_HI_QUALITY) {
    float A = dxt0 * dxt0 + dyt0 * dyt0;
    float B = -2.0f * (dxt0 * dxt1 + dyt0 * dyt1);
    float C = dxt1 * dxt1 + dyt1 * dyt1;
    float F = A * C - B * B * 0.25f;
    float invF = 1.0f / F;
    A *= invF;
    B *= invF;
    C *= invF;
    float AsubC = A - C;
    float R = sqrtf(AsubC * AsubC + B * B);
    rho = sqrtf(2.0f / (A + C - R));
  } else {
    float dxz = 0.0f * 1.0f, dyz = 0.0f * 1.0f;
    float t0 = 0.0f;
    t0 += dxt0 * dxt0;
    t0 += dxt1 * dxt1;
    t0 += dxz * dxz;
    float t1 = 0.0f;
    t1 += dyt0 * dyt0;
    t1 += dyt1 * dyt1;
    t1 += dyz * dyz;
    float lx = len_sqrt(t0);
    float ly = len_sqrt(t1);
    rho = smax(lx, ly);
  }
  if (rho == 0.0f) rho = 0.000001f;
  return fast_log2(rho) + bias;
}

// sampler::calc_anisotropic_info (sampler.cpp:875-958)
__device__ inline void calc_af(dev_sampler const& s, float dxu, float dxv, float dyu, float dyv, float bias,
                               af_info& out) {
  float fw = static_cast<float>(s.width), fh = static_cast<float>(s.height);
  float dxt0 = dxu * fw, dxt1 = dxv * fh, dyt0 = dyu * fw, dyt1 = dyv * fh;
  float ddx_len = len2(dxt0, dxt1);
  float ddy_len = len2(dyt0, dyt1);
  float diag0 = len2(dxt0 - dyt0, dxt1 - dyt1);
  float diag1 = len2(dxt0 + dyt0, dxt1 + dyt1);
  float minor = smin(smin(diag0, diag1), smin(ddx_len, ddy_len));
  if (minor == 0.0f) minor = 0.000001f;
  float long_len, la0, la1;
  if (ddx_len > ddy_len) {
    long_len = ddx_len;
    la0 = dxt0;
    la1 = dxt1;
  } else {
    long_len = ddy_len;
    la0 = dyt0;
    la1 = dyt1;
  }
  float probe_count = (2.0f * long_len / minor) - 1.0f;
  float rounded = fast_round(probe_count);
  rounded = smin(static_cast<float>(s.max_anisotropy), rounded);
  if (rounded < probe_count) minor = 2.0f * long_len / (rounded + 1.0f);
  out.lod = fast_log2(minor) + bias;
  out.probe_count = rounded;
  if (rounded <= 1.0f) {
    out.du = out.dv = 0.0f;
    out.weight_D = 0.0f;
  } else {
    float r = minor / long_len;
    float k = 1.0f - r;
    float inv = 1.0f / (rounded - 1.0f);
    float d0 = ((la0 * k) * 2.0f) * inv;
    float d1 = ((la1 * k) * 2.0f) * inv;
    float d2 = ((0.0f * k) * 2.0f) * inv;
    float d3 = ((0.0f * k) * 2.0f) * inv;
    float l2 = 0.0f;
    l2 += d0 * d0;
    l2 += d1 * d1;
    l2 += d2 * d2;
    l2 += d3 * d3;
    out.weight_D = 256.0f * l2 * 0.25f / (long_len * long_len);
    out.du = d0 / fw;
    out.dv = d1 / fh;
  }
}

// Whether the sampler's texels are 8-bit RGBA / BGRA and both axes wrap:
// the state whose linear lookups take surface_bilinear_wrap8.
__device__ inline bool wrap8_state(dev_sampler const& s) {
  return (s.fmt == SG_FMT_RGBA8 || s.fmt == SG_FMT_BGRA8) && s.address_u == SG_ADDRESS_WRAP &&
         s.address_v == SG_ADDRESS_WRAP;
}

// sample_surface's linear filter for that state, inline: the same
// addressing and interpolation steps without the per-lookup dispatch on
// filter, address mode and format.
__device__ __forceinline__ v4 surface_bilinear_wrap8(dev_sampler const& s, int level, float x, float y) {
  dev_level const lv = s.lv[level];
  int const w = lv.w, h = lv.h;
  int x0, x1, y0, y1;
  float tx, ty;
  wrap_linear(x, w, x0, x1, tx);
  wrap_linear(y, h, y0, y1, ty);
  bool const ok = x0 >= 0 && x1 >= 0 && y0 >= 0 && y1 >= 0 && x0 < w && x1 < w && y0 < h && y1 < h;
  if (!ok) return sample_surface(s, level, x, y, SG_FILTER_LINEAR);
  auto texel = [&](int xx, int yy) -> uint8_t const* { return lv.data + (static_cast<size_t>(yy) * w + xx) * 4; };
  return lerp_2d_unorm8(s.fmt == SG_FMT_RGBA8, texel(x0, y0), texel(x1, y0), texel(x0, y1), texel(x1, y1), tx, ty);
}

// One surface lookup of sample_impl; WRAP8: the sampler is in wrap8_state.
template <bool WRAP8>
__device__ __forceinline__ v4 surface_lookup(dev_sampler const& s, int level, float x, float y, uint32_t filter) {
  if (WRAP8 && filter == SG_FILTER_LINEAR) return surface_bilinear_wrap8(s, level, x, y);
  return sample_surface(s, level, x, y, filter);
}

// sampler::sample_impl<false> (sampler.cpp:680-764)
template <bool WRAP8>
__device__ __forceinline__ v4 sample_impl_t(dev_sampler const& s, float cx, float cy, float miplevel, af_info const* af) {
  int max_lod = 0, min_lod = s.nlevels - 1;
  bool is_mag = (s.mip_filter == SG_FILTER_POINT) ? (miplevel < 0.5f) : (miplevel < 0.0f);
  if (is_mag) return surface_lookup<WRAP8>(s, max_lod, cx, cy, s.mag_filter);
  if (s.mip_filter == SG_FILTER_POINT) {
    int ml = fast_roundi_f(miplevel);  // floor(0.5 + m) with the floori bias: equal for every float
    ml = iclamp(ml, max_lod, min_lod);
    return surface_lookup<WRAP8>(s, ml, cx, cy, s.min_filter);
  }
  // a lookup without anisotropy parameters (tex2d, tex2dlod, sampler::sample)
  // on an anisotropic sampler takes the linear mip path: the reference reads
  // the absent parameters there (sampler.cpp:730-755)
  if (s.mip_filter == SG_FILTER_LINEAR || !af) {
    int lo = fast_floori_f(miplevel);
    int hi = lo + 1;
    float frac = miplevel - static_cast<float>(lo);
    int lc = iclamp(lo, max_lod, min_lod), hc = iclamp(hi, max_lod, min_lod);
    v4 c0 = surface_lookup<WRAP8>(s, lc, cx, cy, s.min_filter);
    v4 c1 = surface_lookup<WRAP8>(s, hc, cx, cy, s.min_filter);
    return mk4(lerp1(c0.x, c1.x, frac), lerp1(c0.y, c1.y, frac), lerp1(c0.z, c1.z, frac), lerp1(c0.w, c1.w, frac));
  }
  float start = -0.5f * (af->probe_count - 1.0f);
  float sx = cx + af->du * start;
  float sy = cy + af->dv * start;
  int lo = fast_roundi_f(miplevel);
  // clamp(size_t(lo), max_lod, min_lod): a negative lo becomes a huge size_t
  int lvl = lo < 0 ? min_lod : (lo > min_lod ? min_lod : lo);
  v4 color = mk4(0, 0, 0, 0);
  float wsum = 0.0f;
  int pc = static_cast<int>(af->probe_count);
  for (int i = -pc + 1; i < pc; i += 2) {
    v4 c0 = surface_lookup<WRAP8>(s, lvl, sx, sy, s.min_filter);
    int widx = static_cast<int>(static_cast<float>(i * i) * af->weight_D);
    float w = c_ewa[widx < 0 ? 0 : (widx > 255 ? 255 : widx)];
    color = color + c0 * w;
    wsum += w;
    sx += af->du;
    sy += af->dv;
  }
  float inv = 1.0f / wsum;
  return color * inv;
}
static __device__ __noinline__ v4 sample_impl(dev_sampler const& s, float cx, float cy, float miplevel, af_info const* af) {
  return wrap8_state(s) ? sample_impl_t<true>(s, cx, cy, miplevel, af) : sample_impl_t<false>(s, cx, cy, miplevel, af);
}
// The same, called (INL false) or inlined into the caller (INL true): a call
// keeps the caller's register count down at the cost of the registers saved
// around it; inlined, the caller gets registers for both.
template <bool INL>
__device__ __forceinline__ v4 sample_impl_sel(dev_sampler const& s, float cx, float cy, float miplevel,
                                              af_info const* af) {
  if constexpr (INL)
    return wrap8_state(s) ? sample_impl_t<true>(s, cx, cy, miplevel, af) : sample_impl_t<false>(s, cx, cy, miplevel, af);
  else
    return sample_impl(s, cx, cy, miplevel, af);
}

__device__ inline float calc_lod_2d(dev_sampler const& s, float dxu, float dxv, float dyu, float dyv) {
  if (s.mip_filter == SG_FILTER_ANISOTROPIC && s.max_anisotropy > 1) {
    af_info af;
    calc_af(s, dxu, dxv, dyu, dyv, 0.0f, af);
    return af.lod;
  }
  return calc_lod(s, dxu, dxv, dyu, dyv, 0.0f);
}

// sampler::sample_cube (sampler.cpp:771-829): the major axis picks the face
// (cubemap_faces order +x -x +y -y +z -z) and its coordinates; the lookup is
// sample_impl<true> on that face.  The reference's cube textures keep the LOD
// range [0, 0], so every lookup reads level 0: the magnification filter
// below the mip threshold, else the minification filter (the linear mip
// blend of level 0 with itself).  A cube sampler must be bound to a cube
// texture (a 2D texture has face 0 only: other faces read face 0 here).
__device__ inline v4 sample_cube(dev_sampler const& s, float x, float y, float z, float miplevel) {
  float const ax = fabsf(x), ay = fabsf(y), az = fabsf(z);
  float sc, tc, m;
  int face;
  if (ax > ay && ax > az) {
    m = ax;
    if (x > 0) {
      sc = 0.5f * (z / m + 1.0f);
      tc = 0.5f * (y / m + 1.0f);
      face = 0;
    } else {
      sc = 0.5f * (-z / m + 1.0f);
      tc = 0.5f * (y / m + 1.0f);
      face = 1;
    }
  } else if (ay > ax && ay > az) {
    m = ay;
    if (y > 0) {
      sc = 0.5f * (x / m + 1.0f);
      tc = 0.5f * (z / m + 1.0f);
      face = 2;
    } else {
      sc = 0.5f * (x / m + 1.0f);
      tc = 0.5f * (-z / m + 1.0f);
      face = 3;
    }
  } else {
    m = az;
    if (z > 0) {
      sc = 0.5f * (-x / m + 1.0f);
      tc = 0.5f * (y / m + 1.0f);
      face = 4;
    } else {
      sc = 0.5f * (x / m + 1.0f);
      tc = 0.5f * (y / m + 1.0f);
      face = 5;
    }
  }
  if (!s.cube) face = 0;
  bool const is_mag = (s.mip_filter == SG_FILTER_POINT) ? (miplevel < 0.5f) : (miplevel < 0.0f);
  if (is_mag) return surface_lookup<false>(s, face, sc, tc, s.mag_filter);
  v4 const c0 = surface_lookup<false>(s, face, sc, tc, s.min_filter);
  if (s.mip_filter == SG_FILTER_POINT) return c0;
  float const frac = miplevel - static_cast<float>(fast_floori_f(miplevel));
  return mk4(lerp1(c0.x, c0.x, frac), lerp1(c0.y, c0.y, frac), lerp1(c0.z, c0.z, frac), lerp1(c0.w, c0.w, frac));
}

template <bool INL = false>
__device__ inline v4 sample_2d_grad(dev_sampler const& s, float u, float v, float dxu, float dxv, float dyu,
                                    float dyv, float bias) {
  af_info af{0, 0, 0, 0, 0};
  float lod;
  if (s.mip_filter == SG_FILTER_ANISOTROPIC && s.max_anisotropy > 1) {
    calc_af(s, dxu, dxv, dyu, dyv, bias, af);
    lod = af.lod;
  } else {
    lod = calc_lod(s, dxu, dxv, dyu, dyv, bias);
  }
  return sample_impl_sel<INL>(s, u, v, lod, &af);
}

}  // namespace sg
