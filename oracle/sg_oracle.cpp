// sg_oracle.cpp -- CPU restatement of Salvia's rasterization pipeline.
//
// ORACLE / TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg load this library; the product path never does.
//
// It exports the same C ABI as the product (include/salvia_gb300.h) so one
// scene script drives both.  It is a single-threaded, op-for-op restatement of
// the reference's CPU renderer; every function names the reference lines it
// follows.  Float expressions keep the reference's operation order and are
// compiled with -ffp-contract=off (no fused multiply-add), which is the
// canonical semantics of the reference built by GCC (x86-64 SSE or aarch64).
// It is pinned against the reference itself (oracle/_ref, built from the
// reference's own sources) through the golden fixtures in tests/golden/.
//
// Results do not depend on the reference's thread count: each 64x64 tile is
// owned by one thread and its primitive list is sorted into API order
// (rasterizer.cpp:947-994), and the vertex caches only deduplicate
// deterministic vertex-shader results (default_vertex_cache.cpp:354-390).
//
// Extensions the reference does not have (each marked EXTENSION below):
// RGBA16F colour, D32F and D24S8 depth formats, and draws without a
// depth-stencil target.
#include "salvia_gb300.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// eflib numerics (eflib/include/eflib/math/math.h:21-164)
inline bool eq_eps(float a, float b) {  // equal<float>, math.h:21-26
  return std::fabs(a - b) <= std::numeric_limits<float>::epsilon();
}
inline float fast_round(float val) {  // math.h:112-126
  uint32_t n;
  std::memcpy(&n, &val, 4);
  uint32_t bias_i = ((23u + 127u) << 23) + (n & 0x80000000u);
  float bias;
  std::memcpy(&bias, &bias_i, 4);
  float f = val;
  f += bias;
  f -= bias;
  return f;
}
inline float fast_floor(float val) {  // math.h:133-136
  float f = fast_round(val);
  return (f > val) ? f - 1 : f;
}
inline int fast_roundi(double d) { return static_cast<int>(std::floor(d + 0.5)); }  // math.h:139-141
const double ROUND_EPS = (0.5f - 1.5e-8);                                          // math.h:155
inline int fast_ceili(double d) { return fast_roundi(d + ROUND_EPS); }             // math.h:154-158
inline int fast_floori(double d) { return fast_roundi(d - ROUND_EPS); }            // math.h:160-164
inline float fast_log2(float val) {                                                // math.h:89-105
  int32_t x;
  std::memcpy(&x, &val, 4);
  int log_2 = ((x >> 23) & 255) - 128;
  x &= ~(255 << 23);
  x += 127 << 23;
  float f;
  std::memcpy(&f, &x, 4);
  f = ((-1.0f / 3) * f + 2) * f - 2.0f / 3;
  return f + log_2;
}
inline uint32_t fbits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}
inline float bitsf(uint32_t u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}
// SSE semantics used by the reference's intrinsic code paths.
inline float sse_max(float a, float b) { return a > b ? a : b; }  // _mm_max_ps: b on NaN
inline float sse_min(float a, float b) { return a < b ? a : b; }  // _mm_min_ps: b on NaN
inline int32_t cvtt(float f) {                                     // _mm_cvttps_epi32
  if (!(f > -2147483904.0f && f < 2147483648.0f)) return INT32_MIN;
  return static_cast<int32_t>(f);
}
inline int32_t cvt_rne(float f) {  // _mm_cvtps_epi32 (round-to-nearest-even)
  if (!(f > -2147483904.0f && f < 2147483648.0f)) return INT32_MIN;
  return static_cast<int32_t>(std::nearbyint(f));
}

struct vec4 {
  float v[4];
  float& operator[](int i) { return v[i]; }
  float operator[](int i) const { return v[i]; }
};
inline vec4 mk(float a, float b, float c, float d) { return vec4{{a, b, c, d}}; }
inline vec4 add(vec4 const& a, vec4 const& b) {
  return mk(a[0] + b[0], a[1] + b[1], a[2] + b[2], a[3] + b[3]);
}
inline vec4 sub(vec4 const& a, vec4 const& b) {
  return mk(a[0] - b[0], a[1] - b[1], a[2] - b[2], a[3] - b[3]);
}
inline vec4 mul(vec4 const& a, float s) { return mk(a[0] * s, a[1] * s, a[2] * s, a[3] * s); }
inline vec4 mulv(vec4 const& a, vec4 const& b) {
  return mk(a[0] * b[0], a[1] * b[1], a[2] * b[2], a[3] * b[3]);
}
inline float dot4(vec4 const& a, vec4 const& b) {  // eflib/src/math.cpp:43-45
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3];
}
inline float len2(float x, float y) {  // vector_::length on a vec2 (vector_generic.h:118-126)
  float t = 0.0f;
  t += x * x;
  t += y * y;
  return static_cast<float>(::sqrt(static_cast<double>(t)));
}

// ---------------------------------------------------------------------------
// pixel formats (salvia/include/salvia/common/colors.h:148-458)
size_t elem_size(uint32_t fmt) {
  switch (fmt) {
  case SG_FMT_RGBA32F: return 16;
  case SG_FMT_RGB32F: return 12;
  case SG_FMT_BGRA8:
  case SG_FMT_RGBA8:
  case SG_FMT_R32F:
  case SG_FMT_R32I:
  case SG_FMT_D32F:
  case SG_FMT_D24S8: return 4;
  case SG_FMT_RG32F:
  case SG_FMT_RGBA16F: return 8;
  default: return 0;
  }
}

// EXTENSION: IEEE binary16 round-to-nearest-even conversion for RGBA16F.
uint16_t f32_to_f16(float f) {
  uint32_t x = fbits(f);
  uint32_t sign = (x >> 16) & 0x8000u;
  uint32_t exp = (x >> 23) & 0xFFu;
  uint32_t man = x & 0x7FFFFFu;
  if (exp == 0xFF) return static_cast<uint16_t>(sign | 0x7C00u | (man ? 0x200u : 0u));
  int32_t e = static_cast<int32_t>(exp) - 127 + 15;
  if (e >= 31) return static_cast<uint16_t>(sign | 0x7C00u);
  if (e <= 0) {
    if (e < -10) return static_cast<uint16_t>(sign);
    man |= 0x800000u;
    uint32_t shift = static_cast<uint32_t>(14 - e);
    uint32_t half = man >> shift;
    uint32_t rem = man & ((1u << shift) - 1u);
    uint32_t mid = 1u << (shift - 1);
    if (rem > mid || (rem == mid && (half & 1u))) ++half;
    return static_cast<uint16_t>(sign | half);
  }
  uint32_t half = (static_cast<uint32_t>(e) << 10) | (man >> 13);
  uint32_t rem = man & 0x1FFFu;
  if (rem > 0x1000u || (rem == 0x1000u && (half & 1u))) ++half;
  return static_cast<uint16_t>(sign | half);
}
float f16_to_f32(uint16_t h) {
  uint32_t sign = (h & 0x8000u) << 16;
  uint32_t exp = (h >> 10) & 0x1Fu;
  uint32_t man = h & 0x3FFu;
  if (exp == 0) {
    if (man == 0) return bitsf(sign);
    float f = static_cast<float>(man) * (1.0f / 16777216.0f);
    return sign ? -f : f;
  }
  if (exp == 31) return bitsf(sign | 0x7F800000u | (man << 13));
  return bitsf(sign | ((exp + 112u) << 23) | (man << 13));
}

// color_rgba8::to_rgba32f (colors.h:176-179)
inline vec4 unorm8_to_f(uint8_t r, uint8_t g, uint8_t b, uint8_t a) {
  const float inv_255 = 1.0f / 255;
  return mk(r * inv_255, g * inv_255, b * inv_255, a * inv_255);
}
// color_rgba8::assign, SSE path (colors.h:182-192)
inline uint8_t f_to_unorm8(float c) {
  float m = c * 255.0f;
  m = sse_max(m, 0.0f);
  m = sse_min(m, 255.0f);
  return static_cast<uint8_t>(cvt_rne(m) & 0xFF);
}

vec4 read_texel(uint32_t fmt, uint8_t const* p) {  // to_rgba32f per format
  switch (fmt) {
  case SG_FMT_RGBA32F: {
    vec4 r;
    std::memcpy(r.v, p, 16);
    return r;
  }
  case SG_FMT_RGB32F: {
    float f[3];
    std::memcpy(f, p, 12);
    return mk(f[0], f[1], f[2], 1.0f);
  }
  case SG_FMT_BGRA8: return unorm8_to_f(p[2], p[1], p[0], p[3]);
  case SG_FMT_RGBA8: return unorm8_to_f(p[0], p[1], p[2], p[3]);
  case SG_FMT_R32F: {
    float f;
    std::memcpy(&f, p, 4);
    return mk(f, 0.0f, 0.0f, 0.0f);
  }
  case SG_FMT_RG32F: {
    float f[2];
    std::memcpy(f, p, 8);
    return mk(f[0], f[1], 0.0f, 0.0f);
  }
  case SG_FMT_R32I: {
    int32_t i;
    std::memcpy(&i, p, 4);
    return mk(static_cast<float>(i), 0.0f, 0.0f, 0.0f);
  }
  case SG_FMT_RGBA16F: {
    uint16_t h[4];
    std::memcpy(h, p, 8);
    return mk(f16_to_f32(h[0]), f16_to_f32(h[1]), f16_to_f32(h[2]), f16_to_f32(h[3]));
  }
  default: return mk(0, 0, 0, 0);
  }
}

void write_texel(uint32_t fmt, uint8_t* p, vec4 const& c) {  // from_rgba32f per format
  switch (fmt) {
  case SG_FMT_RGBA32F: std::memcpy(p, c.v, 16); break;
  case SG_FMT_RGB32F: std::memcpy(p, c.v, 12); break;
  case SG_FMT_BGRA8:
    p[0] = f_to_unorm8(c[2]);
    p[1] = f_to_unorm8(c[1]);
    p[2] = f_to_unorm8(c[0]);
    p[3] = f_to_unorm8(c[3]);
    break;
  case SG_FMT_RGBA8:
    p[0] = f_to_unorm8(c[0]);
    p[1] = f_to_unorm8(c[1]);
    p[2] = f_to_unorm8(c[2]);
    p[3] = f_to_unorm8(c[3]);
    break;
  case SG_FMT_R32F: std::memcpy(p, c.v, 4); break;
  case SG_FMT_RG32F: std::memcpy(p, c.v, 8); break;
  case SG_FMT_R32I: {  // color_r32i::assign (colors.h:301-304)
    int32_t i = static_cast<int32_t>(c[0] + 0.5f);
    std::memcpy(p, &i, 4);
    break;
  }
  case SG_FMT_RGBA16F: {
    uint16_t h[4] = {f32_to_f16(c[0]), f32_to_f16(c[1]), f32_to_f16(c[2]), f32_to_f16(c[3])};
    std::memcpy(p, h, 8);
    break;
  }
  default: break;
  }
}

// Bilinear lerp of four texels (the lerp_2d table, colors.h:340-458).
vec4 lerp4(vec4 const& c0, vec4 const& c1, vec4 const& c2, vec4 const& c3, float tx, float ty) {
  vec4 r;
  for (int i = 0; i < 4; ++i) {
    float c01 = c0[i] + (c1[i] - c0[i]) * tx;
    float c23 = c2[i] + (c3[i] - c2[i]) * tx;
    r[i] = c01 + (c23 - c01) * ty;
  }
  return r;
}
vec4 lerp_2d(uint32_t fmt, uint8_t const* a, uint8_t const* b, uint8_t const* c, uint8_t const* d,
             float tx, float ty) {
  switch (fmt) {
  case SG_FMT_RGBA8:
  case SG_FMT_BGRA8: {  // lerps in 0..255 space, then * (1/255) (colors.h:382-447)
    int ir = fmt == SG_FMT_RGBA8 ? 0 : 2, ib = fmt == SG_FMT_RGBA8 ? 2 : 0;
    auto ld = [&](uint8_t const* p) {
      return mk(static_cast<float>(p[ir]), static_cast<float>(p[1]), static_cast<float>(p[ib]),
                static_cast<float>(p[3]));
    };
    vec4 r = lerp4(ld(a), ld(b), ld(c), ld(d), tx, ty);
    return mul(r, 1.0f / 255);
  }
  case SG_FMT_RGB32F: {  // colors.h:361-370 (keeps the reference's use of c0.r)
    vec4 c0 = read_texel(fmt, a), c1 = read_texel(fmt, b), c2 = read_texel(fmt, c),
         c3 = read_texel(fmt, d);
    float r01 = c0[0] + (c1[0] - c0[0]) * tx, g01 = c0[0] + (c1[1] - c0[1]) * tx,
          b01 = c0[0] + (c1[2] - c0[2]) * tx;
    float r23 = c2[0] + (c3[0] - c2[0]) * tx, g23 = c2[0] + (c3[1] - c2[1]) * tx,
          b23 = c2[0] + (c3[2] - c2[2]) * tx;
    return mk(r01 + (r23 - r01) * ty, r01 + (g23 - g01) * ty, r01 + (b23 - b01) * ty, 1.0f);
  }
  case SG_FMT_RG32F: {  // colors.h:467-475
    vec4 c0 = read_texel(fmt, a), c1 = read_texel(fmt, b), c2 = read_texel(fmt, c),
         c3 = read_texel(fmt, d);
    float r01 = c0[0] + (c1[0] - c0[0]) * tx, g01 = c0[0] + (c1[1] - c0[1]) * tx;
    float r23 = c2[0] + (c3[0] - c2[0]) * tx, g23 = c2[0] + (c3[1] - c2[1]) * tx;
    return mk(r01 + (r23 - r01) * ty, r01 + (g23 - g01) * ty, 0.0f, 0.0f);
  }
  case SG_FMT_R32F:
  case SG_FMT_R32I: {
    vec4 c0 = read_texel(fmt, a), c1 = read_texel(fmt, b), c2 = read_texel(fmt, c),
         c3 = read_texel(fmt, d);
    float r01 = c0[0] + (c1[0] - c0[0]) * tx;
    float r23 = c2[0] + (c3[0] - c2[0]) * tx;
    return mk(r01 + (r23 - r01) * ty, 0.0f, 0.0f, 0.0f);
  }
  default:
    return lerp4(read_texel(fmt, a), read_texel(fmt, b), read_texel(fmt, c), read_texel(fmt, d), tx,
                 ty);
  }
}

// ---------------------------------------------------------------------------
// surfaces and textures (surface.cpp, texture2d.cpp)
struct surface {
  uint32_t w = 0, h = 0, samples = 1, fmt = 0;
  size_t esz = 0;
  std::vector<uint8_t> data;
  surface(uint32_t w_, uint32_t h_, uint32_t s_, uint32_t f_)
    : w(w_), h(h_), samples(s_), fmt(f_), esz(elem_size(f_)) {
    data.resize(size_t(w) * h * samples * esz);
  }
  uint8_t* addr(size_t x, size_t y, size_t s) {  // surface.cpp:277-295
    return data.data() + ((y * w + x) * samples + s) * esz;
  }
  uint8_t const* addr(size_t x, size_t y, size_t s) const {
    return data.data() + ((y * w + x) * samples + s) * esz;
  }
  vec4 get(size_t x, size_t y, size_t s) const { return read_texel(fmt, addr(x, y, s)); }
  void set(size_t x, size_t y, size_t s, vec4 const& c) { write_texel(fmt, addr(x, y, s), c); }
};

struct texture {
  std::vector<std::unique_ptr<surface>> levels;  // level 0 finest (texture.h:17-80)
  uint32_t width = 0, height = 0;
  bool cube = false;  // texture_cube (texture.h:91-102): levels are the six faces, LOD range [0, 0]
};

// surface::make_mip_surface(filter) (surface.cpp:53-92)
std::unique_ptr<surface> make_mip(surface const& src, uint32_t filter) {
  uint32_t mw = (src.w + 1) / 2, mh = (src.h + 1) / 2;
  auto ret = std::make_unique<surface>(mw, mh, src.samples, src.fmt);
  for (uint32_t y = 0; y < mh; ++y) {
    for (uint32_t x = 0; x < mw; ++x) {
      for (uint32_t s = 0; s < src.samples; ++s) {
        if (filter == SG_FILTER_POINT) {
          ret->set(x, y, s, src.get(x * 2, y * 2, s));
        } else {
          // Odd sizes read one texel past the row/column, as the reference
          // does; the read is clamped here to stay inside the allocation.
          uint32_t x1 = std::min(x * 2 + 1, src.w - 1), y1 = std::min(y * 2 + 1, src.h - 1);
          vec4 c0 = src.get(x * 2, y * 2, s), c1 = src.get(x1, y * 2, s),
               c2 = src.get(x * 2, y1, s), c3 = src.get(x1, y1, s);
          vec4 sum = add(add(add(c0, c1), c2), c3);
          ret->set(x, y, s, mul(sum, 0.25f));
        }
      }
    }
  }
  return ret;
}

// texture::calc_lod_limit (texture.h:26-36)
uint32_t lod_limit(uint32_t w, uint32_t h) {
  uint32_t m = std::max(w, std::max(h, 1u)), r = 0;
  while (m > 0) {
    m >>= 1;
    ++r;
  }
  return r;
}

// ---------------------------------------------------------------------------
// sampler (salvia/src/resource/sampler.cpp)
struct sampler {
  sg_sampler_desc d{};
  texture const* tex = nullptr;
};

// The reference's addressers take the SSE (non-EFLIB_NO_SIMD) paths.
// wrap::do_coordi_linear_2d, one axis (sampler.cpp:67-95)
void wrap_linear(float coord, int size, int& lo, int& hi, float& frac) {
  float c0 = coord - static_cast<float>(cvtt(coord));
  float fs = static_cast<float>(size);
  c0 = fs * c0;
  c0 = c0 - 0.5f;
  float ip = static_cast<float>(cvtt(c0));
  if (ip > c0) ip = ip - 1.0f;
  frac = c0 - ip;
  float big = fs * 8192.0f;
  float a0 = ip + 0.0f, a1 = ip + 1.0f;
  a0 = a0 + big;
  a1 = a1 + big;
  float d0 = static_cast<float>(cvtt(a0 / fs)), d1 = static_cast<float>(cvtt(a1 / fs));
  lo = cvtt(a0 - d0 * fs);
  hi = cvtt(a1 - d1 * fs);
}
// mirror::do_coordi_linear_2d (sampler.cpp:168-202)
void mirror_linear(float coord, int size, int& lo, int& hi, float& frac) {
  int sel = fast_floori(coord);
  float o = ((sel & 1) ? 1 + sel - coord : coord - sel) * size - 0.5f;
  float ip = static_cast<float>(cvtt(o));
  if (ip > o) ip = ip - 1.0f;
  frac = o - ip;
  float fs = static_cast<float>(size) - 1.0f;
  float a0 = ip + 0.0f, a1 = ip + 1.0f;
  lo = cvtt(sse_min(sse_max(a0, 0.0f), fs));
  hi = cvtt(sse_min(sse_max(a1, 0.0f), fs));
}
// clamp::do_coordi_linear_2d (sampler.cpp:264-292)
void clamp_linear(float coord, int size, int& lo, int& hi, float& frac) {
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
// border::do_coordi_linear_2d (sampler.cpp:352-391)
void border_linear(float coord, int size, int& lo, int& hi, float& frac) {
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
// Point addressing, do_coordi_point_2d per mode (sampler.cpp:27-47,131-157,226-249,320-350)
int wrap_point(float coord, int size) {
  float c = coord - static_cast<float>(cvtt(coord));
  float fs = static_cast<float>(size);
  c = fs * c;
  float ip = static_cast<float>(cvtt(c));
  if (ip > c) ip = ip - 1.0f;
  float a = ip + fs * 8192.0f;
  float dv = static_cast<float>(cvtt(a / fs));
  return cvtt(a - dv * fs);
}
int mirror_point(float coord, int size) {
  int sel = fast_floori(coord);
  float o = ((sel & 1) ? 1 + sel - coord : coord - sel) * size;
  float ip = static_cast<float>(cvtt(o));
  if (ip > o) ip = ip - 1.0f;
  float fs = static_cast<float>(size) - 1.0f;
  return cvtt(sse_min(sse_max(ip, 0.0f), fs));
}
int clamp_point(float coord, int size) {
  float fs = static_cast<float>(size);
  float c = coord * fs;
  c = sse_max(c, 0.5f);
  c = sse_min(c, fs - 0.5f);
  float ip = static_cast<float>(cvtt(c));
  if (ip > c) ip = ip - 1.0f;
  return cvtt(sse_min(sse_max(ip, 0.0f), fs - 1.0f));
}
int border_point(float coord, int size) {
  float fs = static_cast<float>(size);
  float t = coord * fs;
  t = sse_max(t, -0.5f);
  float c = sse_min(t, fs - -0.5f);
  float ip = static_cast<float>(cvtt(c));
  if (ip > c) ip = ip - 1.0f;
  int ci = cvtt(ip);
  return ci >= size ? -1 : ci;
}
// Scalar (1-D) addressers used when u and v modes differ (sampler.cpp:21-25,124-130,221-225,
// 315-319) via coord_calculator::point_cc / linear_cc (sampler.cpp:396-410).
float coordf(uint32_t mode, float coord, int size) {
  switch (mode) {
  case SG_ADDRESS_WRAP: return (coord - fast_floor(coord)) * size - 0.5f;
  case SG_ADDRESS_MIRROR: {
    int sel = fast_floori(coord);
    return ((sel & 1) ? 1 + sel - coord : coord - sel) * size - 0.5f;
  }
  case SG_ADDRESS_CLAMP: return std::clamp(coord * size, 0.5f, size - 0.5f) - 0.5f;
  default: return std::clamp(coord * size, -0.5f, size + 0.5f) - 0.5f;
  }
}
int coordi_1d(uint32_t mode, int coord, int size) {
  switch (mode) {
  case SG_ADDRESS_WRAP: return (size * 8192 + coord) % size;
  case SG_ADDRESS_MIRROR:
  case SG_ADDRESS_CLAMP: return std::clamp(coord, 0, size - 1);
  default: return coord >= size ? -1 : coord;
  }
}

// surface_sampler::point / linear (sampler.cpp:423-483)
vec4 sample_surface(sampler const& sp, surface const& s, float x, float y, uint32_t filter) {
  int w = static_cast<int>(s.w), h = static_cast<int>(s.h);
  uint32_t mu = sp.d.address_u, mv = sp.d.address_v;
  if (filter == SG_FILTER_POINT) {
    int ix, iy;
    bool two_d = (mu == mv);
    if (two_d) {
      auto pt = [&](float c, int sz) {
        switch (mu) {
        case SG_ADDRESS_WRAP: return wrap_point(c, sz);
        case SG_ADDRESS_MIRROR: return mirror_point(c, sz);
        case SG_ADDRESS_CLAMP: return clamp_point(c, sz);
        default: return border_point(c, sz);
        }
      };
      ix = pt(x, w);
      iy = pt(y, h);
      if (0 <= ix && ix < w && 0 <= iy && iy < h) return s.get(ix, iy, 0);
      vec4 b;
      std::memcpy(b.v, sp.d.border_color, 16);
      return b;
    }
    ix = coordi_1d(mu, fast_floori(coordf(mu, x, w) + 0.5f), w);
    iy = coordi_1d(mv, fast_floori(coordf(mv, y, h) + 0.5f), h);
    if (ix < 0 || iy < 0) {
      vec4 b;
      std::memcpy(b.v, sp.d.border_color, 16);
      return b;
    }
    return s.get(ix, iy, 0);
  }
  int x0, x1, y0, y1;
  float tx, ty;
  if (mu == mv) {
    auto lin = [&](float c, int sz, int& lo, int& hi, float& fr) {
      switch (mu) {
      case SG_ADDRESS_WRAP: wrap_linear(c, sz, lo, hi, fr); break;
      case SG_ADDRESS_MIRROR: mirror_linear(c, sz, lo, hi, fr); break;
      case SG_ADDRESS_CLAMP: clamp_linear(c, sz, lo, hi, fr); break;
      default: border_linear(c, sz, lo, hi, fr); break;
      }
    };
    lin(x, w, x0, x1, tx);
    lin(y, h, y0, y1, ty);
  } else {
    float ox = coordf(mu, x, w);
    int ixp = fast_floori(ox);
    x0 = coordi_1d(mu, ixp, w);
    x1 = coordi_1d(mu, ixp + 1, w);
    tx = ox - ixp;
    float oy = coordf(mv, y, h);
    int iyp = fast_floori(oy);
    y0 = coordi_1d(mv, iyp, h);
    y1 = coordi_1d(mv, iyp + 1, h);
    ty = oy - iyp;
  }
  // Border addressing yields -1 for texels outside; the reference then
  // forms an out-of-range address (surface::get_texel has no check).  The
  // restatement reads the border colour's storage in that case instead.
  auto at = [&](int xx, int yy) -> uint8_t const* {
    if (xx < 0 || yy < 0 || xx >= w || yy >= h) return nullptr;
    return s.addr(xx, yy, 0);
  };
  uint8_t const* a[4] = {at(x0, y0), at(x1, y0), at(x0, y1), at(x1, y1)};
  if (!a[0] || !a[1] || !a[2] || !a[3]) {
    std::vector<uint8_t> tmp(s.esz);
    vec4 b;
    std::memcpy(b.v, sp.d.border_color, 16);
    write_texel(s.fmt, tmp.data(), b);
    for (auto& p : a)
      if (!p) p = tmp.data();
    return lerp_2d(s.fmt, a[0], a[1], a[2], a[3], tx, ty);
  }
  return lerp_2d(s.fmt, a[0], a[1], a[2], a[3], tx, ty);
}

struct af_info {
  float lod = 0, probe_count = 0, weight_D = 0;
  float du = 0, dv = 0;
};

// EWA weight table: (exp(a*r) - exp(a)) / (1 - exp(a)), a = -2, r = i/255,
// printed to six significant digits (sampler.cpp:629-678; the reference
// comments it as Blender's table).  Regenerated here from the formula.
float const* ewa_table() {
  static float tab[256];
  static bool init = false;
  if (!init) {
    for (int i = 0; i < 256; ++i) {
      double r = i / 255.0;
      double v = (std::exp(-2.0 * r) - std::exp(-2.0)) / (1.0 - std::exp(-2.0));
      char buf[32];
      std::snprintf(buf, sizeof(buf), "%.6g", v);
      tab[i] = std::strtof(buf, nullptr);
    }
    tab[0] = 1.0f;
    tab[255] = 0.0f;
    init = true;
  }
  return tab;
}

// sampler::calc_lod (sampler.cpp:521-603)
float calc_lod(sampler const& sp, uint32_t sw, uint32_t sh, vec4 const& ddx, vec4 const& ddy,
               float bias) {
  vec4 size = mk(static_cast<float>(sw), static_cast<float>(sh), 1.0f, 0.0f);
  if (sp.d.mip_quality == SG_MIP_LO_QUALITY) {
    vec4 maxd = mk(std::max(std::fabs(ddx[0]), std::fabs(ddy[0])),
                   std::max(std::fabs(ddx[1]), std::fabs(ddy[1])),
                   std::max(std::fabs(ddx[2]), std::fabs(ddy[2])), 0.0f);
    maxd = mulv(maxd, size);
    float rho = std::max(std::max(maxd[0], maxd[1]), maxd[2]);
    return fast_log2(rho) + bias;
  }
  vec4 dxt = mulv(ddx, size), dyt = mulv(ddy, size);
  float rho;
  if (sp.d.mip_quality == SG_MIP_HI_QUALITY) {
    float A = dxt[0] * dxt[0] + dyt[0] * dyt[0];
    float B = -2.0f * (dxt[0] * dxt[1] + dyt[0] * dyt[1]);
    float Cc = dxt[1] * dxt[1] + dyt[1] * dyt[1];
    float F = A * Cc - B * B * 0.25f;
    float invF = 1.0f / F;
    A *= invF;
    B *= invF;
    Cc *= invF;
    float AsubC = A - Cc;
    float R = std::sqrt(AsubC * AsubC + B * B);
    rho = std::sqrt(2.0f / (A + Cc - R));
  } else {
    // ddx_ts.xyz().length(): sqrt in double of the float sum (vector_generic.h:118-126)
    float t0 = 0.0f;
    t0 += dxt[0] * dxt[0];
    t0 += dxt[1] * dxt[1];
    t0 += dxt[2] * dxt[2];
    float t1 = 0.0f;
    t1 += dyt[0] * dyt[0];
    t1 += dyt[1] * dyt[1];
    t1 += dyt[2] * dyt[2];
    float lx = static_cast<float>(::sqrt(static_cast<double>(t0)));
    float ly = static_cast<float>(::sqrt(static_cast<double>(t1)));
    rho = std::max(lx, ly);
  }
  if (rho == 0.0f) rho = 0.000001f;
  return fast_log2(rho) + bias;
}

// sampler::calc_anisotropic_info (sampler.cpp:875-958)
void calc_af(sampler const& sp, uint32_t sw, uint32_t sh, vec4 const& ddx, vec4 const& ddy,
             float bias, af_info& out) {
  float fw = static_cast<float>(sw), fh = static_cast<float>(sh);
  vec4 size = mk(fw, fh, 1.0f, 0.0f);
  vec4 dxt = mulv(ddx, size), dyt = mulv(ddy, size);
  float ddx_len = len2(dxt[0], dxt[1]);
  float ddy_len = len2(dyt[0], dyt[1]);
  vec4 dm = sub(dxt, dyt), dp = add(dxt, dyt);
  float diag0 = len2(dm[0], dm[1]);
  float diag1 = len2(dp[0], dp[1]);
  float minor = std::min(std::min(diag0, diag1), std::min(ddx_len, ddy_len));
  if (minor == 0.0f) minor = 0.000001f;
  vec4 const* long_axis;
  float long_len;
  if (ddx_len > ddy_len) {
    long_len = ddx_len;
    long_axis = &dxt;
  } else {
    long_len = ddy_len;
    long_axis = &dyt;
  }
  float probe_count = (2.0f * long_len / minor) - 1.0f;
  float rounded = fast_round(probe_count);
  rounded = std::min(static_cast<float>(sp.d.max_anisotropy), rounded);
  if (rounded < probe_count) minor = 2.0f * long_len / (rounded + 1.0f);
  out.lod = fast_log2(minor) + bias;
  out.probe_count = rounded;
  if (rounded <= 1.0f) {
    out.du = out.dv = 0.0f;
    out.weight_D = 0.0f;
  } else {
    float r = minor / long_len;
    float k = (1.0f - r);
    vec4 delta = mul(mul(mul(*long_axis, k), 2.0f), 1.0f / (rounded - 1.0f));
    float l2 = 0.0f;  // delta_uv.length_sqr() over 4 components
    l2 += delta[0] * delta[0];
    l2 += delta[1] * delta[1];
    l2 += delta[2] * delta[2];
    l2 += delta[3] * delta[3];
    out.weight_D = static_cast<float>(255 + 1) * l2 * 0.25f / (long_len * long_len);
    out.du = delta[0] / fw;
    out.dv = delta[1] / fh;
  }
}

// sampler::sample_impl<false> (sampler.cpp:680-764)
vec4 sample_impl(sampler const& sp, float cx, float cy, float miplevel, af_info const* af) {
  texture const& t = *sp.tex;
  int max_lod = 0, min_lod = t.cube ? 0 : static_cast<int>(t.levels.size()) - 1;
  bool is_mag = (sp.d.mip_filter == SG_FILTER_POINT) ? (miplevel < 0.5f) : (miplevel < 0.0f);
  if (is_mag) return sample_surface(sp, *t.levels[max_lod], cx, cy, sp.d.mag_filter);
  if (sp.d.mip_filter == SG_FILTER_POINT) {
    int ml = fast_floori(0.5 + miplevel);
    ml = std::clamp(ml, max_lod, min_lod);
    return sample_surface(sp, *t.levels[ml], cx, cy, sp.d.min_filter);
  }
  // EXTENSION: a lookup without anisotropy parameters (tex2d, tex2dlod,
  // sampler::sample) on an anisotropic sampler takes the linear mip path;
  // the reference reads the absent parameters there (sampler.cpp:730-755)
  if (sp.d.mip_filter == SG_FILTER_LINEAR || !af) {
    int lo = fast_floori(miplevel);
    int hi = lo + 1;
    float frac = miplevel - lo;
    int lc = std::clamp(lo, max_lod, min_lod), hc = std::clamp(hi, max_lod, min_lod);
    vec4 c0 = sample_surface(sp, *t.levels[lc], cx, cy, sp.d.min_filter);
    vec4 c1 = sample_surface(sp, *t.levels[hc], cx, cy, sp.d.min_filter);
    vec4 r;  // salvia::lerp(color_rgba32f, color_rgba32f, t), SSE path (colors.h:309-320)
    for (int i = 0; i < 4; ++i) r[i] = c0[i] + (c1[i] - c0[i]) * frac;
    return r;
  }
  // anisotropic
  float start = -0.5f * (af->probe_count - 1.0f);
  float sx = cx + af->du * start;
  float sy = cy + af->dv * start;
  int lo = fast_roundi(miplevel);
  size_t lo_sz = std::clamp(static_cast<size_t>(lo), static_cast<size_t>(max_lod),
                            static_cast<size_t>(min_lod));
  float const* ewa = ewa_table();
  vec4 color = mk(0, 0, 0, 0);
  float wsum = 0.0f;
  int pc = static_cast<int>(af->probe_count);
  for (int i = -pc + 1; i < pc; i += 2) {
    vec4 c0 = sample_surface(sp, *t.levels[lo_sz], sx, sy, sp.d.min_filter);
    float w = ewa[static_cast<int>(i * i * af->weight_D)];
    color = add(color, mul(c0, w));
    wsum += w;
    sx += af->du;
    sy += af->dv;
  }
  float inv = 1 / wsum;  // vector_::operator/= multiplies by the reciprocal
  return mul(color, inv);
}

// sampler::sample_cube (sampler.cpp:771-829): the major axis picks the face
// and its coordinates, then sample_impl<true> on that face with the cube's
// LOD range [0, 0] (texture_cube sets none): level 0, the magnification
// filter below the mip threshold, else the minification filter (a linear mip
// blends level 0 with itself).  EXTENSION: the anisotropic mip filter, whose
// parameters the reference reads from a null pointer here, takes the
// linear path.
vec4 sample_cube(sampler const& sp, float x, float y, float z, float miplevel) {
  float ax = std::fabs(x), ay = std::fabs(y), az = std::fabs(z);
  float s, t, m;
  int face;
  if (ax > ay && ax > az) {
    m = ax;
    if (x > 0) { s = 0.5f * (z / m + 1.0f); t = 0.5f * (y / m + 1.0f); face = 0; }
    else { s = 0.5f * (-z / m + 1.0f); t = 0.5f * (y / m + 1.0f); face = 1; }
  } else if (ay > ax && ay > az) {
    m = ay;
    if (y > 0) { s = 0.5f * (x / m + 1.0f); t = 0.5f * (z / m + 1.0f); face = 2; }
    else { s = 0.5f * (x / m + 1.0f); t = 0.5f * (-z / m + 1.0f); face = 3; }
  } else {
    m = az;
    if (z > 0) { s = 0.5f * (-x / m + 1.0f); t = 0.5f * (y / m + 1.0f); face = 4; }
    else { s = 0.5f * (x / m + 1.0f); t = 0.5f * (y / m + 1.0f); face = 5; }
  }
  texture const& tx = *sp.tex;
  surface const& f = *tx.levels[tx.cube ? face : 0];
  bool is_mag = (sp.d.mip_filter == SG_FILTER_POINT) ? (miplevel < 0.5f) : (miplevel < 0.0f);
  if (is_mag) return sample_surface(sp, f, s, t, sp.d.mag_filter);
  vec4 c0 = sample_surface(sp, f, s, t, sp.d.min_filter);
  if (sp.d.mip_filter == SG_FILTER_POINT) return c0;
  int lo = fast_floori(miplevel);
  float frac = miplevel - lo;
  vec4 r;
  for (int k = 0; k < 4; ++k) r[k] = c0[k] + (c0[k] - c0[k]) * frac;  // lerp(c0, c1 = c0, frac)
  return r;
}

float calc_lod_2d(sampler const& sp, float dxu, float dxv, float dyu, float dyv) {
  uint32_t sw = sp.tex->width, sh = sp.tex->height;
  vec4 ddx = mk(dxu, dxv, 0, 0), ddy = mk(dyu, dyv, 0, 0);
  if (sp.d.mip_filter == SG_FILTER_ANISOTROPIC && sp.d.max_anisotropy > 1) {
    af_info af;
    calc_af(sp, sw, sh, ddx, ddy, 0.0f, af);
    return af.lod;
  }
  return calc_lod(sp, sw, sh, ddx, ddy, 0.0f);
}

vec4 sample_2d_grad(sampler const& sp, float u, float v, float dxu, float dxv, float dyu,
                    float dyv, float bias) {
  uint32_t sw = sp.tex->width, sh = sp.tex->height;
  vec4 ddx = mk(dxu, dxv, 0, 0), ddy = mk(dyu, dyv, 0, 0);
  af_info af;
  float lod;
  if (sp.d.mip_filter == SG_FILTER_ANISOTROPIC && sp.d.max_anisotropy > 1) {
    calc_af(sp, sw, sh, ddx, ddy, bias, af);
    lod = af.lod;
  } else {
    lod = calc_lod(sp, sw, sh, ddx, ddy, bias);
  }
  return sample_impl(sp, u, v, lod, &af);
}

// ---------------------------------------------------------------------------
// vertex-shader output registers (shader_regs.h:32-86)
constexpr int MAX_REGS = 1 + SG_MAX_VARYINGS;
struct vso {
  vec4 r[MAX_REGS];
  vec4& pos() { return r[0]; }
  vec4 const& pos() const { return r[0]; }
};

struct draw_ctx;

// ---------------------------------------------------------------------------
struct device_state {
  std::vector<sg_shader_module const*> user_shaders;  // program SG_USER_PROGRAM_BASE + i
  uint32_t next = 1;
  std::map<uint32_t, std::vector<uint8_t>> buffers;
  std::map<uint32_t, std::unique_ptr<texture>> textures;
  std::map<uint32_t, sampler> samplers;
};

constexpr int TILE = 64;  // rasterizer.cpp:32

struct tri_info {  // triangle_info (shader_regs.h:93-104)
  vso const* v0 = nullptr;
  bool front = false;
  float bbox[4];
  vec4 edge[3];
  vso ddx, ddy;
};

struct draw_ctx {
  device_state* dev;
  sg_draw_desc const* d;
  surface* color = nullptr;
  surface* more[SG_MAX_COLOR_TARGETS - 1] = {};  // colour targets 1..
  uint32_t nmore = 0;
  surface* ds = nullptr;
  uint32_t nattr = 0;
  uint32_t mods[SG_MAX_VARYINGS];
  bool has_centroid = false;
  uint32_t samples = 1;
  float sp[4][2];
  uint64_t full_mask = 1, quad_full_mask = 0;
  float target_w = 0, target_h = 0;
  bool early_z = false;
  sampler const* vs_samp = nullptr;
  sampler const* ps_samp = nullptr;
  sg_draw_stats stats{};
  mutable bool front = false;  // the triangle being rasterised faces front (rasterizer.cpp:915)
};

// stream_assembler::fetch_vertex / get_vec4 (stream_assembler.cpp:26-93)
void fetch_vertex(draw_ctx const& c, uint32_t index, vec4* regs) {
  sg_draw_desc const& d = *c.d;
  for (uint32_t r = 0; r < d.num_inputs; ++r) {
    sg_vs_input const& in = d.inputs[r];
    sg_vertex_stream const& st = d.streams[in.slot];
    auto const& buf = c.dev->buffers.at(st.buffer);
    size_t off = size_t(in.offset) + size_t(st.stride) * index + st.offset;
    float f[4] = {0, 0, 0, 0};
    size_t n = 4;
    switch (in.format) {
    case SG_VFMT_R32_FLOAT: n = 1; break;
    case SG_VFMT_R32G32_FLOAT: n = 2; break;
    case SG_VFMT_R32G32B32_FLOAT: n = 3; break;
    default: n = 4; break;
    }
    if (off + n * 4 <= buf.size()) std::memcpy(f, buf.data() + off, n * 4);
    float dw = in.semantic == SG_SEMANTIC_POSITION ? 1.0f : 0.0f;
    if (n < 4) f[3] = dw;
    regs[r] = mk(f[0], f[1], f[2], f[3]);
  }
}

// eflib::transform(out, v, m): out[j] = dot_prod4(v, column j) (eflib/src/math.cpp:142-154)
vec4 transform(vec4 const& v, float const* m) {
  vec4 o;
  for (int j = 0; j < 4; ++j) o[j] = dot4(v, mk(m[0 + j], m[4 + j], m[8 + j], m[12 + j]));
  return o;
}

vec4 sample_level0(sampler const& sp, float u, float v) {  // sampler::sample(u, v, 0)
  return sample_impl(sp, u, v, 0.0f, nullptr);
}

// sampler::sample for a user vertex body's vertex texture fetch
void uvs_sample(void* b, float u, float v, float lod, float out[4]) {
  sampler const* sp = static_cast<draw_ctx const*>(b)->vs_samp;
  if (!sp) {  // no sampler in the slot: zeros (as on the device)
    for (int k = 0; k < 4; ++k) out[k] = 0.0f;
    return;
  }
  vec4 const r = sample_impl(*sp, u, v, lod, nullptr);
  for (int k = 0; k < 4; ++k) out[k] = r[k];
}

void run_vs(draw_ctx const& c, uint32_t index, vso& out) {
  vec4 in[SG_MAX_VS_INPUTS];
  for (auto& x : in) x = mk(0, 0, 0, 0);
  fetch_vertex(c, index, in);
  sg_shader const& s = c.d->vs;
  if (s.program >= SG_USER_PROGRAM_BASE) {  // a user vertex shader's host body
    sg_shader_module const* m = c.dev->user_shaders[s.program - SG_USER_PROGRAM_BASE];
    sg_host_vs_io io{};
    for (int r = 0; r < SG_MAX_VS_INPUTS; ++r)
      for (int k = 0; k < 4; ++k) io.in[r][k] = in[r][k];
    io.num_varyings = c.nattr;
    io.constants = s.constants;
    io.backend = const_cast<draw_ctx*>(&c);
    io.sample = uvs_sample;
    m->host_vs(&io);
    out.pos() = mk(io.position[0], io.position[1], io.position[2], io.position[3]);
    for (uint32_t i = 0; i < c.nattr; ++i) out.r[1 + i] = mk(io.attr[i][0], io.attr[i][1], io.attr[i][2], io.attr[i][3]);
    return;
  }
  switch (s.program) {
  case SG_VS_TRANSFORM:
    out.pos() = transform(in[0], s.constants);
    for (uint32_t i = 0; i < c.nattr; ++i) out.r[1 + i] = in[i + 1];
    break;
  case SG_VS_MORPH_DISPLACE: {
    vec4 p = add(in[0], mul(sub(in[1], in[0]), s.constants[16]));
    vec4 n = in[2];
    float h = sample_level0(*c.vs_samp, in[3][0], in[3][1])[0];
    float hs = h * s.constants[17];
    p[0] = p[0] + n[0] * hs;
    p[1] = p[1] + n[1] * hs;
    p[2] = p[2] + n[2] * hs;
    out.pos() = transform(p, s.constants);
    if (c.nattr > 0) out.r[1] = in[3];
    if (c.nattr > 1) out.r[2] = n;
    break;
  }
  default: out.pos() = mk(0, 0, 0, 1); break;
  }
}

// index_fetcher::fetch_indexes for one primitive (index_fetcher.cpp:26-115)
void fetch_indexes(draw_ctx const& c, uint32_t prim, uint32_t out[3]) {
  sg_draw_desc const& d = *c.d;
  uint32_t ids[3];
  if (d.topology == SG_TOPOLOGY_LINE_LIST || d.topology == SG_TOPOLOGY_LINE_STRIP) {
    // index_fetcher.cpp:53-60; the third index is unused
    ids[0] = d.topology == SG_TOPOLOGY_LINE_LIST ? prim * 2 : prim;
    ids[1] = ids[0] + 1;
    ids[2] = ids[1];
  } else if (d.topology == SG_TOPOLOGY_TRIANGLE_STRIP) {
    ids[0] = prim + 0;
    ids[1] = prim + 1;
    ids[2] = prim + 2;
    if (prim & 1) std::swap(ids[0], ids[2]);
  } else {
    ids[0] = prim * 3 + 0;
    ids[1] = prim * 3 + 1;
    ids[2] = prim * 3 + 2;
  }
  if (d.indexed) {
    auto const& ib = c.dev->buffers.at(d.index_buffer);
    uint32_t stride = d.index_format == SG_INDEX_U16 ? 2 : 4;
    uint8_t const* base = ib.data() + size_t(d.start) * stride;
    for (int i = 0; i < 3; ++i) {
      uint32_t v;
      if (stride == 2) {
        uint16_t s;
        std::memcpy(&s, base + size_t(ids[i]) * 2, 2);
        v = s;
      } else {
        std::memcpy(&v, base + size_t(ids[i]) * 4, 4);
      }
      out[i] = v + static_cast<uint32_t>(d.base_vertex);
    }
  } else {
    // renderer_impl::draw sets base_vertex = 0 (renderer_impl.cpp:337-344)
    for (int i = 0; i < 3; ++i) out[i] = ids[i];
  }
}

// cull functions (raster_state.cpp:10-32)
bool cull(draw_ctx const& c, float area) {
  uint32_t cm = c.d->raster.cull_mode;
  bool ccw = c.d->raster.front_ccw != 0;
  if (cm == SG_CULL_NONE) return false;
  bool cull_ccw = (cm == SG_CULL_FRONT) ? ccw : !ccw;  // cull_front: ccw?ccw:cw; back: ccw?cw:ccw
  return cull_ccw ? (area <= 0) : (area >= 0);
}

// vs_output_op lerp_n (shader.cpp:170-180)
void vso_lerp(draw_ctx const& c, vso& out, vso const& a, vso const& b, float t) {
  out.pos() = add(a.pos(), mul(sub(b.pos(), a.pos()), t));
  for (uint32_t i = 0; i < c.nattr; ++i) {
    out.r[1 + i] = a.r[1 + i];
    if (!(c.mods[i] & SG_AM_NOINTERPOLATION))
      out.r[1 + i] = add(out.r[1 + i], mul(sub(b.r[1 + i], a.r[1 + i]), t));
  }
}

float clip_dot(int plane, vec4 const& p) {  // planes_ (clipper.cpp:21-27) with dot_prod4
  static const vec4 planes[2] = {mk(0.0f, 0.0f, 1.0f, 0.0f), mk(0.0f, 0.0f, -1.0f, 1.0f)};
  return dot4(planes[plane], p);
}

// clipper::clip_solid_triangle + clip_triangle_to_poly_general (clipper.cpp:43-228).
// Returns the output triangles' vertex pointers (3 per triangle).
void clip_triangle(draw_ctx const& c, vso* tv[3], std::vector<std::unique_ptr<vso>>& pool,
                   std::vector<vso*>& out) {
  bool in_frustum = true;
  for (int p = 0; p < 2 && in_frustum; ++p)
    for (int v = 0; v < 3; ++v)
      if (clip_dot(p, tv[v]->pos()) < 0) {
        in_frustum = false;
        break;
      }
  if (in_frustum) {
    // compute_front (clipper.cpp:91-100)
    float pv[3][2];
    for (int i = 0; i < 3; ++i) {
      float iw = 1.0f / tv[i]->pos()[3];
      pv[i][0] = tv[i]->pos()[0] * iw;
      pv[i][1] = tv[i]->pos()[1] * iw;
    }
    float ax = pv[2][0] - pv[0][0], ay = pv[2][1] - pv[0][1];
    float bx = pv[1][0] - pv[0][0], by = pv[1][1] - pv[0][1];
    float area = ax * by - ay * bx;
    bool front = area > 0.0f;
    if (cull(c, front ? 1.0f : -1.0f)) return;
    int off = front ? 0 : 1;
    out.push_back(tv[0]);
    out.push_back(tv[1 + off]);
    out.push_back(tv[2 - off]);
    return;
  }
  vso* cv[2][5];
  uint32_t n[2];
  cv[0][0] = tv[0];
  cv[0][1] = tv[1];
  cv[0][2] = tv[2];
  n[0] = 3;
  float dd[2] = {0, 0};
  int src = 0, dst = 1;
  bool is_front = false;
  for (int p = 0; p < 2; ++p) {
    n[dst] = 0;
    if (n[src] != 0) dd[0] = clip_dot(p, cv[src][0]->pos());
    for (uint32_t i = 0, j = 1; i < n[src]; ++i, ++j) {
      j %= n[src];
      dd[1] = clip_dot(p, cv[src][j]->pos());
      if (dd[0] >= 0.0f) {
        cv[dst][n[dst]++] = cv[src][i];
        if (dd[1] < 0.0f) {
          pool.push_back(std::make_unique<vso>());
          vso_lerp(c, *pool.back(), *cv[src][i], *cv[src][j], dd[0] / (dd[0] - dd[1]));
          cv[dst][n[dst]++] = pool.back().get();
        }
      } else {
        if (dd[1] >= 0.0f) {
          pool.push_back(std::make_unique<vso>());
          vso_lerp(c, *pool.back(), *cv[src][j], *cv[src][i], dd[1] / (dd[1] - dd[0]));
          cv[dst][n[dst]++] = pool.back().get();
        }
      }
      dd[0] = dd[1];
    }
    if (p == 0 && n[dst] >= 3) {
      float pv[3][2];
      for (int i = 0; i < 3; ++i) {
        vec4 const& q = cv[dst][i]->pos();
        float inv_abs_w = 1 / std::fabs(q[3]);
        pv[i][0] = q[0] * inv_abs_w;
        pv[i][1] = q[1] * inv_abs_w;
      }
      float ax = pv[2][0] - pv[0][0], ay = pv[2][1] - pv[0][1];
      float bx = pv[1][0] - pv[0][0], by = pv[1][1] - pv[0][1];
      float area = ax * by - ay * bx;
      is_front = area > 0.0f;
      if (cull(c, area)) return;
    }
    src = (src + 1) & 1;
    dst = (dst + 1) & 1;
  }
  uint32_t nv = n[src];
  if (nv < 3) return;
  // Fan re-triangulation (clipper.cpp:75-89).  The reference's loop bound
  // writes (n-2)*3-2 triangles of which only the first n-2 are consumed
  // (num_clipped_verts = (n-2)*3); those are the ones produced here.
  for (uint32_t t = 1; t + 1 < nv; ++t) {
    out.push_back(cv[src][0]);
    if (is_front) {
      out.push_back(cv[src][t]);
      out.push_back(cv[src][t + 1]);
    } else {
      out.push_back(cv[src][t + 1]);
      out.push_back(cv[src][t]);
    }
  }
}

// viewport_transform + project_n in place (shader.cpp:499-511, 117-134)
void vp_project(draw_ctx const& c, vso& v) {
  sg_viewport const& vp = c.d->viewport;
  vec4& p = v.pos();
  float invw = eq_eps(p[3], 0.0f) ? 1.0f : 1.0f / p[3];
  vec4 pos = mul(p, invw);
  float ox = (vp.x + vp.w) * 0.5f;
  float oy = (vp.y + vp.h) * 0.5f;
  p[0] = (float(vp.w) * 0.5f) * pos[0] + ox;
  p[1] = (float(vp.h) * 0.5f) * -pos[1] + oy;
  p[2] = (vp.maxz - vp.minz) * pos[2] + vp.minz;
  p[3] = invw;
  for (uint32_t i = 0; i < c.nattr; ++i)
    if (!(c.mods[i] & SG_AM_NOPERSPECTIVE)) v.r[1 + i] = mul(v.r[1 + i], p[3]);
}

// rasterizer::compute_triangle_info (rasterizer.cpp:864-945) with
// compute_derivative_n (shader.cpp:414-449)
void compute_tri(draw_ctx const& c, vso const* verts[3], tri_info& ti) {
  ti.v0 = nullptr;
  vec4 const* vp[3] = {&verts[0]->pos(), &verts[1]->pos(), &verts[2]->pos()};
  double dist[3];
  for (int i = 0; i < 3; ++i)
    dist[i] = std::fabs(static_cast<double>((*vp[i])[0])) + std::fabs(static_cast<double>((*vp[i])[1]));
  int r0;
  if (dist[0] < dist[1])
    r0 = dist[0] < dist[2] ? 0 : 2;
  else
    r0 = dist[1] < dist[2] ? 1 : 2;
  int r1 = (r0 + 1) % 3, r2 = (r1 + 1) % 3;
  vso const* rv[3] = {verts[r0], verts[r1], verts[r2]};
  int nreg = 1 + static_cast<int>(c.nattr);
  vso e01, e02;
  for (int i = 0; i < nreg; ++i) {
    e01.r[i] = sub(rv[1]->r[i], rv[0]->r[i]);
    e02.r[i] = sub(rv[2]->r[i], rv[0]->r[i]);
  }
  float area = e02.r[0][0] * e01.r[0][1] - e02.r[0][1] * e01.r[0][0];  // cross_prod2
  if (eq_eps(area, 0.0f)) return;
  ti.front = area > 0.0f;
  float inv_area = 1.0f / area;
  ti.bbox[0] = std::min(std::min((*vp[0])[0], (*vp[1])[0]), (*vp[2])[0]);
  ti.bbox[1] = std::max(std::max((*vp[0])[0], (*vp[1])[0]), (*vp[2])[0]);
  ti.bbox[2] = std::min(std::min((*vp[0])[1], (*vp[1])[1]), (*vp[2])[1]);
  ti.bbox[3] = std::max(std::max((*vp[0])[1], (*vp[1])[1]), (*vp[2])[1]);
  for (int i = 0; i < 3; ++i) {
    int se = i, ee = (i + 1) % 3;
    ti.edge[i][0] = (*vp[se])[1] - (*vp[ee])[1];
    ti.edge[i][1] = (*vp[ee])[0] - (*vp[se])[0];
    ti.edge[i][2] = (*vp[ee])[0] * (*vp[se])[1] - (*vp[ee])[1] * (*vp[se])[0];
    ti.edge[i][3] = 0.0f;
  }
  float e01x = e01.r[0][0], e01y = e01.r[0][1], e02x = e02.r[0][0], e02y = e02.r[0][1];
  for (int i = 0; i < nreg; ++i) {
    for (int k = 0; k < 4; ++k) {
      float xd = e02.r[i][k] * e01y - e01.r[i][k] * e02y;
      float yd = e01.r[i][k] * e02x - e02.r[i][k] * e01x;
      ti.ddx.r[i][k] = xd * inv_area;
      ti.ddy.r[i][k] = yd * inv_area;
    }
  }
  ti.v0 = rv[0];
}

// ---------------------------------------------------------------------------
// output merger (framebuffer.cpp)
bool cmp(uint32_t f, float a, float b) {
  switch (f) {
  case SG_CMP_NEVER: return false;
  case SG_CMP_LESS: return a < b;
  case SG_CMP_EQUAL: return a == b;
  case SG_CMP_LESS_EQUAL: return a <= b;
  case SG_CMP_GREATER: return a > b;
  case SG_CMP_NOT_EQUAL: return a != b;
  case SG_CMP_GREATER_EQUAL: return a >= b;
  default: return true;
  }
}
bool cmpu(uint32_t f, uint32_t a, uint32_t b) {
  switch (f) {
  case SG_CMP_NEVER: return false;
  case SG_CMP_LESS: return a < b;
  case SG_CMP_EQUAL: return a == b;
  case SG_CMP_LESS_EQUAL: return a <= b;
  case SG_CMP_GREATER: return a > b;
  case SG_CMP_NOT_EQUAL: return a != b;
  case SG_CMP_GREATER_EQUAL: return a >= b;
  default: return true;
  }
}
uint32_t sop(uint32_t op, uint32_t ref, uint32_t cur) {  // framebuffer.cpp:136-166
  switch (op) {
  case SG_SOP_KEEP: return cur;
  case SG_SOP_ZERO: return 0;
  case SG_SOP_REPLACE: return ref;
  case SG_SOP_INCR_SAT: return std::min<uint32_t>(0xFF, cur + 1);
  case SG_SOP_DECR_SAT: return std::max<uint32_t>(0, cur - 1);
  case SG_SOP_INVERT: return ~cur;
  case SG_SOP_INCR_WRAP: return (cur + 1) & 0xFF;
  case SG_SOP_DECR_WRAP: return (cur - 1 + 256) & 0xFF;
  default: return cur;
  }
}

// EXTENSION: 24-bit unorm depth quantisation for D24S8.
inline uint32_t d24_quantize(float z) {
  float c = std::min(std::max(z, 0.0f), 1.0f) * 16777215.0f;
  return static_cast<uint32_t>(std::nearbyint(c));
}

struct ds_rw {  // depth/stencil read/write function selection (framebuffer.cpp:358-425)
  bool read_depth = false, write_depth = false, stencil = false;
};

ds_rw ds_functions(draw_ctx const& c) {
  ds_rw f;
  sg_depth_stencil_desc const& s = c.d->depth_stencil;
  if (!c.ds) return f;
  if (s.depth_enable) {
    f.read_depth = s.depth_func != SG_CMP_NEVER && s.depth_func != SG_CMP_ALWAYS;
    f.write_depth = s.depth_write && s.depth_func != SG_CMP_NEVER;
  }
  f.stencil = s.stencil_enable != 0;
  if (c.ds->fmt == SG_FMT_D32F) f.stencil = false;
  return f;
}

// Reads depth (and stencil masked by the read mask) of one sample.  For
// RG32F: depth in .r, stencil bits in .g (framebuffer.cpp:38-86).
void ds_read(draw_ctx const& c, ds_rw const& f, size_t x, size_t y, size_t s, float& depth,
             uint32_t& q, uint32_t& stencil) {
  depth = 0.0f;
  stencil = 0;
  q = 0;
  uint8_t const* p = c.ds->addr(x, y, s);
  uint32_t rm = c.d->depth_stencil.stencil_read_mask & 0xFFu;  // uint8_t in depth_stencil_desc
  switch (c.ds->fmt) {
  case SG_FMT_RG32F:
    if (f.read_depth) std::memcpy(&depth, p, 4);
    if (f.stencil) {
      std::memcpy(&stencil, p + 4, 4);
      stencil &= rm;
    }
    break;
  case SG_FMT_D32F:
    if (f.read_depth) std::memcpy(&depth, p, 4);
    break;
  case SG_FMT_D24S8: {
    uint32_t w;
    std::memcpy(&w, p, 4);
    if (f.read_depth) q = w & 0xFFFFFFu;
    if (f.stencil) stencil = (w >> 24) & rm;
    break;
  }
  default: break;
  }
}
void ds_write(draw_ctx const& c, ds_rw const& f, size_t x, size_t y, size_t s, float depth,
              uint32_t stencil, uint32_t wmask) {
  uint8_t* p = c.ds->addr(x, y, s);
  switch (c.ds->fmt) {
  case SG_FMT_RG32F:
    if (f.write_depth) std::memcpy(p, &depth, 4);
    if (f.stencil) {
      uint32_t v = stencil & wmask;
      std::memcpy(p + 4, &v, 4);
    }
    break;
  case SG_FMT_D32F:
    if (f.write_depth) std::memcpy(p, &depth, 4);
    break;
  case SG_FMT_D24S8: {
    uint32_t w;
    std::memcpy(&w, p, 4);
    if (f.write_depth) w = (w & 0xFF000000u) | d24_quantize(depth);
    if (f.stencil) w = (w & 0x00FFFFFFu) | ((stencil & wmask & 0xFFu) << 24);
    std::memcpy(p, &w, 4);
    break;
  }
  default: break;
  }
}
bool depth_test(draw_ctx const& c, ds_rw const& f, float depth, float old_depth, uint32_t old_q) {
  uint32_t func = c.d->depth_stencil.depth_enable ? c.d->depth_stencil.depth_func : SG_CMP_ALWAYS;
  if (c.ds && c.ds->fmt == SG_FMT_D24S8 && f.read_depth) return cmpu(func, d24_quantize(depth), old_q);
  return cmp(func, depth, old_depth);
}

struct rasterizer_state {
  draw_ctx* c;
  std::vector<tri_info> const* tris;
  ds_rw f;
  sg_draw_stats* st;
};

// cpp_blend_shader programs (shader.h:209-215)
// `more`: the pixel's colours 1.. (SG_MAX_COLOR_TARGETS - 1 of them)
struct user_bs_backend {
  draw_ctx const* c;
  size_t x, y;
};
surface* user_bs_target(user_bs_backend const& u, uint32_t t) {
  return t == 0 ? u.c->color : t <= u.c->nmore ? u.c->more[t - 1] : nullptr;
}
void ubs_get(void* b, uint32_t t, uint32_t s, float out[4]) {
  auto& u = *static_cast<user_bs_backend*>(b);
  surface* sf = user_bs_target(u, t);
  vec4 v = sf ? sf->get(u.x, u.y, s) : mk(0, 0, 0, 0);
  for (int k = 0; k < 4; ++k) out[k] = v[k];
}
void ubs_set(void* b, uint32_t t, uint32_t s, const float c[4]) {
  auto& u = *static_cast<user_bs_backend*>(b);
  if (surface* sf = user_bs_target(u, t)) sf->set(u.x, u.y, s, mk(c[0], c[1], c[2], c[3]));
}
void blend(draw_ctx const& c, size_t x, size_t y, size_t s, vec4 const& src, vec4 const* more) {
  if (!c.color) return;
  if (c.d->bs.program >= SG_USER_PROGRAM_BASE) {  // a user blend shader's host body
    sg_shader_module const* m = c.dev->user_shaders[c.d->bs.program - SG_USER_PROGRAM_BASE];
    user_bs_backend ub{&c, x, y};
    sg_host_bs_io io{};
    io.sample = static_cast<uint32_t>(s);
    for (int k = 0; k < 4; ++k) io.in_color[0][k] = src[k];
    for (uint32_t t = 0; t + 1 < SG_MAX_COLOR_TARGETS; ++t)
      for (int k = 0; k < 4; ++k) io.in_color[t + 1][k] = more[t][k];
    io.constants = c.d->bs.constants;
    io.backend = &ub;
    io.get = ubs_get;
    io.set = ubs_set;
    m->host_bs(&io);
    return;
  }
  switch (c.d->bs.program) {
  case SG_BS_REPLACE_ALL:  // color(i, s) = in.color[i] for every bound target
    c.color->set(x, y, s, src);
    for (uint32_t i = 0; i < c.nmore; ++i) c.more[i]->set(x, y, s, more[i]);
    break;
  case SG_BS_LERP_SRC_ALPHA: {
    vec4 dst = c.color->get(x, y, s);
    vec4 r;
    for (int i = 0; i < 4; ++i) r[i] = dst[i] + (src[i] - dst[i]) * src[3];
    c.color->set(x, y, s, r);
    break;
  }
  case SG_BS_ADD: c.color->set(x, y, s, add(c.color->get(x, y, s), src)); break;
  default: c.color->set(x, y, s, src); break;
  }
}

// framebuffer::render_sample (framebuffer.cpp:445-479)
void render_sample(rasterizer_state& rs, size_t x, size_t y, size_t s, vec4 const& src,
                   float depth, bool front, vec4 const* more) {
  draw_ctx const& c = *rs.c;
  if (c.early_z || !c.ds) {  // EXTENSION: without a depth-stencil target every sample passes
    blend(c, x, y, s, src, more);
    return;
  }
  sg_depth_stencil_desc const& d = c.d->depth_stencil;
  float old_depth;
  uint32_t old_q, old_stencil;
  ds_read(c, rs.f, x, y, s, old_depth, old_q, old_stencil);
  bool dpass = depth_test(c, rs.f, depth, old_depth, old_q);
  uint32_t ref = rs.f.stencil ? (static_cast<uint32_t>(c.d->stencil_ref) & d.stencil_read_mask & 0xFFu) : 0;
  sg_stencil_face_desc const& face = front ? d.front : d.back;
  bool spass = rs.f.stencil ? cmpu(face.func, ref, old_stencil) : true;
  if (dpass && spass) {
    uint32_t ns = rs.f.stencil ? sop(face.pass_op, ref, old_stencil) : 0;
    blend(c, x, y, s, src, more);
    ds_write(c, rs.f, x, y, s, depth, ns, d.stencil_write_mask & 0xFFu);
  }
}

// framebuffer::early_z_test (framebuffer.cpp:522-590)
uint64_t early_z_px(rasterizer_state& rs, size_t x, size_t y, uint32_t px_mask, float depth,
                    float const* aa) {
  draw_ctx const& c = *rs.c;
  if (c.samples == 1 && px_mask == c.full_mask) {
    float od;
    uint32_t oq, os;
    ds_read(c, rs.f, x, y, 0, od, oq, os);
    if (depth_test(c, rs.f, depth, od, oq)) {
      ds_write(c, rs.f, x, y, 0, depth, 0, 0);
      return 1;
    }
    return 0;
  }
  uint64_t mask = 0;
  for (uint32_t i = 0; i < c.samples; ++i) {
    if (!(px_mask & (1u << i))) continue;
    float od;
    uint32_t oq, os;
    ds_read(c, rs.f, x, y, i, od, oq, os);
    float nd = aa[i] + depth;
    bool pass = depth_test(c, rs.f, nd, od, oq);
    mask |= static_cast<uint64_t>(pass ? 1 : 0) << i;
    if (pass) ds_write(c, rs.f, x, y, i, nd, 0, 0);
  }
  return mask;
}

// framebuffer::render_sample_quad (framebuffer.cpp:481-520)
void render_sample_quad(rasterizer_state& rs, size_t x, size_t y, uint64_t mask, vec4 const* col,
                        vec4 const (*more)[SG_MAX_COLOR_TARGETS - 1], float const* depth, bool front,
                        float const* aa) {
  draw_ctx const& c = *rs.c;
  for (int i = 0; i < 4; ++i) {
    size_t px = x + (i & 1), py = y + ((i & 2) >> 1);
    uint64_t m = mask & 0xFFFF;
    mask >>= 16;
    if (m == 0) continue;
    if (c.samples == 1) {
      render_sample(rs, px, py, 0, col[i], depth[i], front, more[i]);
    } else {
      for (uint32_t s = 0; s < c.samples; ++s)
        if (m & (1u << s)) render_sample(rs, px, py, s, col[i], depth[i] + aa[s], front, more[i]);
    }
  }
}

// A user pixel shader's host body on pixel i of a quad: its registers and
// this restatement's cpp_pixel_shader helpers (cpp_pixel_shader.cpp:13-60).
struct user_ps_backend {
  draw_ctx const* c;
  vso const* quad;
  int i;
};
void ups_reg(vso const& v, uint32_t reg, float out[4]) {
  for (int k = 0; k < 4; ++k) out[k] = v.r[1 + reg][k];
}
void ups_ddx(void* b, uint32_t reg, float out[4]) {
  auto& u = *static_cast<user_ps_backend*>(b);
  vec4 d = sub(u.quad[1].r[1 + reg], u.quad[0].r[1 + reg]);
  for (int k = 0; k < 4; ++k) out[k] = d[k];
}
void ups_ddy(void* b, uint32_t reg, float out[4]) {
  auto& u = *static_cast<user_ps_backend*>(b);
  vec4 d = sub(u.quad[2].r[1 + reg], u.quad[0].r[1 + reg]);
  for (int k = 0; k < 4; ++k) out[k] = d[k];
}
void ups_put(vec4 const& v, float out[4]) {
  for (int k = 0; k < 4; ++k) out[k] = v[k];
}
// a draw without a sampler in the slot samples zeros (as on the device)
bool ups_no_sampler(void* b, float out[4]) {
  if (static_cast<user_ps_backend*>(b)->c->ps_samp) return false;
  for (int k = 0; k < 4; ++k) out[k] = 0.0f;
  return true;
}
void ups_tex2d(void* b, uint32_t reg, float out[4]) {
  if (ups_no_sampler(b, out)) return;
  auto& u = *static_cast<user_ps_backend*>(b);
  vec4 dx = sub(u.quad[1].r[1 + reg], u.quad[0].r[1 + reg]), dy = sub(u.quad[2].r[1 + reg], u.quad[0].r[1 + reg]);
  float lod = calc_lod_2d(*u.c->ps_samp, dx[0], dx[1], dy[0], dy[1]);
  vec4 const& a = u.quad[u.i].r[1 + reg];
  ups_put(sample_impl(*u.c->ps_samp, a[0], a[1], lod, nullptr), out);
}
void ups_tex2dlod(void* b, uint32_t reg, float out[4]) {
  if (ups_no_sampler(b, out)) return;
  auto& u = *static_cast<user_ps_backend*>(b);
  vec4 const& a = u.quad[u.i].r[1 + reg];
  ups_put(sample_impl(*u.c->ps_samp, a[0], a[1], a[3], nullptr), out);
}
void ups_tex2dproj(void* b, uint32_t reg, float out[4]) {
  if (ups_no_sampler(b, out)) return;
  auto& u = *static_cast<user_ps_backend*>(b);
  vec4 const& a = u.quad[u.i].r[1 + reg];
  vec4 nx = add(a, sub(u.quad[1].r[1 + reg], u.quad[0].r[1 + reg]));
  vec4 ny = add(a, sub(u.quad[2].r[1 + reg], u.quad[0].r[1 + reg]));
  auto proj = [](vec4 const& v, int k) { return (v[k] / v[3] + 1.0f) * 0.5f; };
  float px = proj(a, 0), py = proj(a, 1);
  ups_put(sample_2d_grad(*u.c->ps_samp, px, py, proj(nx, 0) - px, proj(nx, 1) - py, proj(ny, 0) - px,
                         proj(ny, 1) - py, 0.0f),
          out);
}
void ups_sample(void* b, float u_, float v, float lod, float out[4]) {
  if (ups_no_sampler(b, out)) return;
  ups_put(sample_impl(*static_cast<user_ps_backend*>(b)->c->ps_samp, u_, v, lod, nullptr), out);
}
void ups_sample_grad(void* b, float u_, float v, float dxu, float dxv, float dyu, float dyv, float out[4]) {
  if (ups_no_sampler(b, out)) return;
  ups_put(sample_2d_grad(*static_cast<user_ps_backend*>(b)->c->ps_samp, u_, v, dxu, dxv, dyu, dyv, 0.0f), out);
}
void ups_sample_cube(void* b, float x, float y, float z, float lod, float out[4]) {
  if (ups_no_sampler(b, out)) return;
  ups_put(sample_cube(*static_cast<user_ps_backend*>(b)->c->ps_samp, x, y, z, lod), out);
}
bool run_user_ps(draw_ctx const& c, vso const* quad, int i, vec4& out, vec4* more) {
  sg_shader_module const* m = c.dev->user_shaders[c.d->ps.program - SG_USER_PROGRAM_BASE];
  user_ps_backend ub{&c, quad, i};
  sg_host_ps_io io{};
  for (uint32_t a = 0; a < SG_MAX_VARYINGS; ++a)
    if (a < c.nattr) ups_reg(quad[i], a, io.attr[a]);
  for (int k = 0; k < 4; ++k) io.position[k] = quad[i].r[0][k];
  io.front_face = c.front ? 1u : 0u;
  io.num_varyings = c.nattr;
  io.constants = c.d->ps.constants;
  io.backend = &ub;
  io.ddx = ups_ddx;
  io.ddy = ups_ddy;
  io.tex2d = ups_tex2d;
  io.tex2dlod = ups_tex2dlod;
  io.tex2dproj = ups_tex2dproj;
  io.sample = ups_sample;
  io.sample_grad = ups_sample_grad;
  io.sample_cube = ups_sample_cube;
  bool const keep = m->host_ps(&io) != 0;
  out = mk(io.color[0][0], io.color[0][1], io.color[0][2], io.color[0][3]);
  for (uint32_t k = 0; k + 1 < SG_MAX_COLOR_TARGETS; ++k)
    more[k] = mk(io.color[k + 1][0], io.color[k + 1][1], io.color[k + 1][2], io.color[k + 1][3]);
  return keep;
}

// cpp_pixel_shader programs; tex2d's LOD is computed once per quad from
// the quad's attribute differences (cpp_pixel_shader.cpp:13-31).
// `more` receives out.color[1..] (zero unless the program writes them).
bool run_ps(draw_ctx const& c, vso const* quad, int i, vec4& out, vec4* more, float& lod_cache, bool& have_lod) {
  sg_shader const& s = c.d->ps;
  vso const& in = quad[i];
  for (uint32_t k = 0; k + 1 < SG_MAX_COLOR_TARGETS; ++k) more[k] = mk(0, 0, 0, 0);
  if (s.program >= SG_USER_PROGRAM_BASE) return run_user_ps(c, quad, i, out, more);
  switch (s.program) {
  case SG_PS_COLOR: out = in.r[1]; return true;
  case SG_PS_COLOR_MRT:  // out.color[k] = in.attr[k]
    out = in.r[1];
    for (uint32_t k = 1; k < c.nattr && k < SG_MAX_COLOR_TARGETS; ++k) more[k - 1] = in.r[1 + k];
    return true;
  case SG_PS_CONSTANT: out = mk(s.constants[0], s.constants[1], s.constants[2], s.constants[3]); return true;
  case SG_PS_TEX_MODULATE: {
    if (!have_lod) {
      vec4 dx = sub(quad[1].r[1], quad[0].r[1]);
      vec4 dy = sub(quad[2].r[1], quad[0].r[1]);
      lod_cache = calc_lod_2d(*c.ps_samp, dx[0], dx[1], dy[0], dy[1]);
      have_lod = true;
    }
    vec4 t = sample_impl(*c.ps_samp, in.r[1][0], in.r[1][1], lod_cache, nullptr);
    out = mulv(t, in.r[2]);
    return true;
  }
  case SG_PS_TEX_GRAD_MODULATE:
  case SG_PS_TEX_GRAD_LEARNED: {  // the oracle of the learned filter is the plain lookup it approximates
    vec4 dx = sub(quad[1].r[1], quad[0].r[1]);
    vec4 dy = sub(quad[2].r[1], quad[0].r[1]);
    vec4 t = sample_2d_grad(*c.ps_samp, in.r[1][0], in.r[1][1], dx[0], dx[1], dy[0], dy[1], 0.0f);
    out = mulv(t, in.r[2]);
    return true;
  }
  case SG_PS_TEX_LOD_MODULATE: {  // tex2dlod: sampler::sample(x, y, w) (cpp_pixel_shader.cpp:33-40)
    vec4 t = sample_impl(*c.ps_samp, in.r[1][0], in.r[1][1], in.r[1][3], nullptr);
    out = mulv(t, in.r[2]);
    return true;
  }
  case SG_PS_TEX_PROJ_MODULATE: {  // tex2dproj (cpp_pixel_shader.cpp:42-60)
    vec4 const& a = in.r[1];
    vec4 nx = add(a, sub(quad[1].r[1], quad[0].r[1]));
    vec4 ny = add(a, sub(quad[2].r[1], quad[0].r[1]));
    auto proj = [](vec4 const& v, int k) { return (v[k] / v[3] + 1.0f) * 0.5f; };
    float px = proj(a, 0), py = proj(a, 1);
    vec4 t = sample_2d_grad(*c.ps_samp, px, py, proj(nx, 0) - px, proj(nx, 1) - py, proj(ny, 0) - px,
                            proj(ny, 1) - py, 0.0f);
    out = mulv(t, in.r[2]);
    return true;
  }
  case SG_PS_TEXCUBE_MODULATE: {  // sampler::sample_cube(x, y, z, w) (sampler.cpp:771-829)
    vec4 const& a = in.r[1];
    out = mulv(sample_cube(*c.ps_samp, a[0], a[1], a[2], a[3]), in.r[2]);
    return true;
  }
  case SG_PS_TEX_ALPHA_TEST: {  // tex2d * attr[1]; discarded below constants[0] alpha
    if (!have_lod) {
      vec4 dx = sub(quad[1].r[1], quad[0].r[1]);
      vec4 dy = sub(quad[2].r[1], quad[0].r[1]);
      lod_cache = calc_lod_2d(*c.ps_samp, dx[0], dx[1], dy[0], dy[1]);
      have_lod = true;
    }
    out = mulv(sample_impl(*c.ps_samp, in.r[1][0], in.r[1][1], lod_cache, nullptr), in.r[2]);
    return !(out[3] < s.constants[0]);
  }
  default: out = mk(0, 0, 0, 0); return true;
  }
}

// cpp_pixel_shader::execute (cpp_pixel_shader.cpp:62-74).  The reference
// builds the quad's pass mask as `(passed ? 0xFFFF : 0) << (i * 16)` with an
// int left operand: the shift of pixel 1 gives the negative int 0xFFFF0000,
// which sign-extends into the 64-bit mask and sets pixels 1-3, and the
// shifts of pixels 2 and 3 by 32 and 48 bits act as shifts by 0 and 16 (the
// 32-bit shift count wraps).  So pixel 0 is kept when pixel 0 or pixel 2
// passes, and pixels 1-3 are all kept when pixel 1 or pixel 3 passes; with
// no discard every pixel is kept.
uint64_t execute_ps(draw_ctx const& c, vso const* quad, vec4* out, vec4 (*more)[SG_MAX_COLOR_TARGETS - 1]) {
  bool pass[4];
  float lod = 0;
  bool have = false;
  for (int i = 0; i < 4; ++i) pass[i] = run_ps(c, quad, i, out[i], more[i], lod, have);
  uint64_t mask = 0;
  if (pass[0] || pass[2]) mask |= 0xFFFFull;
  if (pass[1] || pass[3]) mask |= 0xFFFFFFFFFFFF0000ull;
  return mask;
}

// step_2d_unproj_pos_quad (shader.cpp:257-287)
void pos_quad(vso* px, vso const& in, float s0, vso const& d0, float s1, vso const& d1) {
  vec4 p00;
  for (int k = 0; k < 4; ++k) p00[k] = in.r[0][k] + (d0.r[0][k] * s0 + d1.r[0][k] * s1);
  px[0].r[0] = p00;
  px[1].r[0] = add(p00, d0.r[0]);
  px[2].r[0] = add(p00, d1.r[0]);
  px[3].r[0] = add(px[1].r[0], d1.r[0]);
}
// step_2d_unproj_attr_n_quad (shader.cpp:289-367)
void attr_quad(draw_ctx const& c, vso* px, vso const& in, float s0, vso const& d0, float s1,
               vso const& d1) {
  float invw[4];
  for (int i = 0; i < 4; ++i) invw[i] = 1.0f / px[i].r[0][3];
  for (uint32_t a = 0; a < c.nattr; ++a) {
    int r = 1 + static_cast<int>(a);
    vec4 v[4];
    if (c.mods[a] & SG_AM_NOINTERPOLATION) {
      v[0] = v[1] = v[2] = v[3] = in.r[r];
    } else {
      for (int k = 0; k < 4; ++k) v[0][k] = in.r[r][k] + (d0.r[r][k] * s0 + d1.r[r][k] * s1);
      v[1] = add(v[0], d0.r[r]);
      v[2] = add(v[0], d1.r[r]);
      v[3] = add(v[1], d1.r[r]);
    }
    for (int i = 0; i < 4; ++i)
      px[i].r[r] = (c.mods[a] & SG_AM_NOPERSPECTIVE) ? v[i] : mul(v[i], invw[i]);
  }
}
// step_2d_unproj_attr_n (shader.cpp:208-255), used by the centroid path
void attr_one(draw_ctx const& c, vso& out, vso const& in, float s0, vso const& d0, float s1,
              vso const& d1) {
  float invw = 1.0f / out.r[0][3];
  for (uint32_t a = 0; a < c.nattr; ++a) {
    int r = 1 + static_cast<int>(a);
    vec4 v;
    if (c.mods[a] & SG_AM_NOINTERPOLATION) {
      v = in.r[r];
    } else {
      for (int k = 0; k < 4; ++k) v[k] = in.r[r][k] + (d0.r[r][k] * s0 + d1.r[r][k] * s1);
    }
    out.r[r] = (c.mods[a] & SG_AM_NOPERSPECTIVE) ? v : mul(v, invw);
  }
}

// rasterizer::draw_full_quad / draw_quad (rasterizer.cpp:1245-1421)
void draw_quad(rasterizer_state& rs, tri_info const& ti, uint32_t left, uint32_t top,
               uint64_t quad_mask, bool full, float const* aa) {
  draw_ctx const& c = *rs.c;
  // EXTENSION: pixels outside the render target are not covered.  The
  // reference writes past the row end there (targets whose width or height
  // is not a multiple of 4); for multiple-of-4 sizes this never triggers.
  for (int i = 0; i < 4; ++i) {
    if (left + (i & 1) >= static_cast<uint32_t>(c.target_w) ||
        top + ((i & 2) >> 1) >= static_cast<uint32_t>(c.target_h)) {
      quad_mask &= ~(0xFFFFull << (16 * i));
      full = false;
    }
  }
  if (quad_mask == 0) return;
  vso px[4];
  vso const& v0 = *ti.v0;
  float dx = 0.5f + left - v0.r[0][0];
  float dy = 0.5f + top - v0.r[0][1];
  pos_quad(px, v0, dx, ti.ddx, dy, ti.ddy);
  float depth[4] = {px[0].r[0][2], px[1].r[0][2], px[2].r[0][2], px[3].r[0][2]};
  uint64_t tested = quad_mask;
  if (c.early_z) {
    tested = 0;
    for (int i = 0; i < 4; ++i) {
      uint32_t pm = static_cast<uint32_t>((quad_mask >> (16 * i)) & 0xFFFF);
      if (pm == 0) continue;
      tested |= early_z_px(rs, left + (i & 1), top + ((i & 2) >> 1), pm, depth[i], aa) << (16 * i);
    }
  }
  if (tested == 0) return;
  if (full || !c.has_centroid) {
    attr_quad(c, px, v0, dx, ti.ddx, dy, ti.ddy);
  } else {
    for (int i = 0; i < 4; ++i) {
      int ix = i & 1, iy = (i & 2) >> 1;
      float pdx = dx + ix, pdy = dy + iy;
      uint32_t pm = static_cast<uint32_t>((quad_mask >> (i * 16)) & 0xFFFF);
      if (pm != c.full_mask && pm != 0) {
        float cx = 0, cy = 0;
        int n = 0;
        for (uint32_t s = 0; s < c.samples; ++s)
          if (pm & (1u << s)) {
            cx += c.sp[s][0];
            cy += c.sp[s][1];
            ++n;
          }
        float inv = 1 / static_cast<float>(n);
        cx *= inv;
        cy *= inv;
        pdx += cx - 0.5f;
        pdy += cy - 0.5f;
      }
      attr_one(c, px[i], v0, pdx, ti.ddx, pdy, ti.ddy);
    }
  }
  rs.st->ps_invocations += 4;
  vec4 col[4];
  vec4 colm[4][SG_MAX_COLOR_TARGETS - 1];
  c.front = ti.front;  // cpp_pixel_shader::update_front_face (rasterizer.cpp:692)
  tested &= execute_ps(c, px, col, colm);
  if (full && tested == 0) return;  // draw_full_quad checks the PS-masked value
  rs.st->backend_input_pixels += 4;
  render_sample_quad(rs, left, top, tested, col, colm, depth, ti.front, aa);
}

// rasterizer::draw_partial_tile (rasterizer.cpp:298-439), SSE path
void draw_partial_tile(rasterizer_state& rs, tri_info const& ti, int left, int top,
                       float const* aa) {
  draw_ctx const& c = *rs.c;
  float lf = static_cast<float>(left), tf = static_cast<float>(top);
  float ev[3];
  for (int e = 0; e < 3; ++e) ev[e] = ti.edge[e][2] - (lf * ti.edge[e][0] + tf * ti.edge[e][1]);
  uint32_t pm[16] = {0};
  for (uint32_t s = 0; s < c.samples; ++s) {
    for (int iy = 0; iy < 4; ++iy) {
      float my = c.sp[s][1] + static_cast<float>(iy);
      for (int ix = 0; ix < 4; ++ix) {
        float mx = c.sp[s][0] + static_cast<float>(ix);
        bool rej = false;
        for (int e = 0; e < 3; ++e) {
          float v = mx * ti.edge[e][0] + my * ti.edge[e][1];
          rej = rej || (v < ev[e]);
        }
        if (!rej) pm[iy * 4 + ix] |= 1u << s;
      }
    }
  }
  for (int q = 0; q < 4; ++q) {
    int qx = (q & 1) << 1, qy = q & 2;
    int st = qx | (qy << 2);
    uint64_t m = (uint64_t(pm[st]) & 0xFFFF) | ((uint64_t(pm[st + 1]) & 0xFFFF) << 16) |
                 ((uint64_t(pm[st + 4]) & 0xFFFF) << 32) | ((uint64_t(pm[st + 5]) & 0xFFFF) << 48);
    if (m == 0) continue;
    bool full = (m == c.quad_full_mask);
    draw_quad(rs, ti, left + qx, top + qy, full ? c.quad_full_mask : m, full, aa);
  }
}

// rasterizer::rasterize_triangle + subdivide_tile (rasterizer.cpp:617-773, 441-571)
void rasterize_triangle(rasterizer_state& rs, uint32_t entry, float tile_x, float tile_y) {
  draw_ctx const& c = *rs.c;
  uint32_t prim = entry >> 1, full = entry & 1;
  tri_info const& ti = (*rs.tris)[prim];
  bool mark_x[3], mark_y[3];
  for (int e = 0; e < 3; ++e) {
    mark_x[e] = ti.edge[e][0] > 0;
    mark_y[e] = ti.edge[e][1] > 0;
  }
  float x_min = ti.bbox[0] - tile_x, x_max = ti.bbox[1] - tile_x;
  float y_min = ti.bbox[2] - tile_y, y_max = ti.bbox[3] - tile_y;
  std::vector<uint32_t> reg[2];
  reg[0].push_back(full << 31);
  int src = 0, dst = 1;
  int vpleft0 = fast_floori(tile_x), vptop0 = fast_floori(tile_y);
  uint32_t sub_w = fast_floori(static_cast<float>(TILE)), sub_h = sub_w;
  float step_x[3], step_y[3], r2a[3], pev[3], ev[3];
  for (int e = 0; e < 3; ++e) {
    step_x[e] = TILE * ti.edge[e][0];
    step_y[e] = TILE * ti.edge[e][1];
    r2a[e] = -std::fabs(step_x[e]) - std::fabs(step_y[e]);
    pev[e] = mark_x[e] * TILE * ti.edge[e][0] + mark_y[e] * TILE * ti.edge[e][1];
    ev[e] = ti.edge[e][2] - pev[e];
  }
  float aa[4];
  if (c.samples > 1) {
    for (uint32_t s = 0; s < c.samples; ++s)
      aa[s] = (c.sp[s][0] - 0.5f) * ti.ddx.r[0][2] + (c.sp[s][1] - 0.5f) * ti.ddy.r[0][2];
  } else {
    aa[0] = 0.0f;
  }
  float trr = c.target_w + 0.0f, trb = c.target_h + 0.0f;
  while (!reg[src].empty()) {
    reg[dst].clear();
    sub_w /= 4;
    sub_h /= 4;
    for (int e = 0; e < 3; ++e) {
      step_x[e] *= 0.25f;
      step_y[e] *= 0.25f;
      r2a[e] *= 0.25f;
      pev[e] *= 0.25f;
      ev[e] = ti.edge[e][2] - pev[e];
    }
    for (uint32_t packed : reg[src]) {
      uint32_t rx = packed & 0xFF, ry = (packed >> 8) & 0xFF;
      bool is_full = (packed >> 31) != 0;
      int vpleft = static_cast<int>(std::max(0u, static_cast<unsigned>(vpleft0 + rx)));
      int vptop = static_cast<int>(std::max(0u, static_cast<unsigned>(vptop0 + ry)));
      if (vpleft >= trr || vptop >= trb) continue;
      if (is_full) {
        int vpright = static_cast<int>(std::min(static_cast<uint32_t>(vpleft0) + rx + sub_w * 4,
                                                static_cast<uint32_t>(trr)));
        int vpbottom = static_cast<int>(std::min(static_cast<uint32_t>(vptop0) + ry + sub_h * 4,
                                                 static_cast<uint32_t>(trb)));
        for (int t = vptop; t < vpbottom; t += 2)
          for (int l = vpleft; l < vpright; l += 2)
            draw_quad(rs, ti, static_cast<uint32_t>(l), static_cast<uint32_t>(t),
                      c.quad_full_mask, true, aa);
        continue;
      }
      if (sub_w <= 1 && sub_h <= 1) {
        draw_partial_tile(rs, ti, vpleft, vptop, aa);
        continue;
      }
      // subdivide_tile, SSE path (rasterizer.cpp:458-571)
      float lf = static_cast<float>(vpleft), tf = static_cast<float>(vptop);
      float ev3[3];
      for (int e = 0; e < 3; ++e) ev3[e] = ev[e] - (lf * ti.edge[e][0] + tf * ti.edge[e][1]);
      uint32_t nw = sub_w, nh = sub_h;
      for (int iy = 0; iy < 4; ++iy) {
        for (int ix = 0; ix < 4; ++ix) {
          bool rej = false, acc_fail = false;
          for (int e = 0; e < 3; ++e) {
            float sxv = step_x[e] * static_cast<float>(ix);
            float syv = step_y[e] * static_cast<float>(iy);
            float srej = sxv + syv;
            float sacc = srej + r2a[e];
            rej = rej || (srej < ev3[e]);
            acc_fail = acc_fail || (sacc < ev3[e]);
          }
          int32_t mx = static_cast<int32_t>(rx + nw * ix), my = static_cast<int32_t>(ry + nh * iy);
          rej = rej || (x_min >= static_cast<float>(mx + static_cast<int32_t>(nw))) ||
                (x_max < static_cast<float>(mx)) ||
                (y_min >= static_cast<float>(my + static_cast<int32_t>(nh))) ||
                (y_max < static_cast<float>(my));
          if (!rej) {
            uint32_t code = static_cast<uint32_t>(mx) | (static_cast<uint32_t>(my) << 8) |
                            (acc_fail ? 0u : 0x80000000u);
            reg[dst].push_back(code);
          }
        }
      }
    }
    src = (src + 1) & 1;
    dst = !src;
  }
}

// ---------------------------------------------------------------------------
// Lines and wireframe (the header's definition; the reference stops at
// ef_unimplemented, its rasterize_line in rasterizer.cpp:60-213 holds the
// intended DDA).

// A segment cut at z >= 0, then at z <= w; false when nothing is left.
bool clip_line(draw_ctx const& c, vso*& a, vso*& b, std::vector<std::unique_ptr<vso>>& pool) {
  for (int p = 0; p < 2; ++p) {
    float da = clip_dot(p, a->pos()), db = clip_dot(p, b->pos());
    if (da < 0.0f && db < 0.0f) return false;
    if (da >= 0.0f && db < 0.0f) {
      pool.push_back(std::make_unique<vso>());
      vso_lerp(c, *pool.back(), *a, *b, da / (da - db));
      b = pool.back().get();
    } else if (da < 0.0f && db >= 0.0f) {
      pool.push_back(std::make_unique<vso>());
      vso_lerp(c, *pool.back(), *b, *a, db / (db - da));
      a = pool.back().get();
    }
  }
  return true;
}

// unproject_n (shader.cpp:136-160)
void unproject(draw_ctx const& c, vso& out, vso const& in) {
  float inv_w = 1.0f / in.pos()[3];
  out.pos() = in.pos();
  for (uint32_t i = 0; i < c.nattr; ++i)
    out.r[1 + i] = (c.mods[i] & SG_AM_NOPERSPECTIVE) ? in.r[1 + i] : mul(in.r[1 + i], inv_w);
}

// lerp_n on every register (shader.cpp:171-180)
void lerp_regs(draw_ctx const& c, vso& out, vso const& a, vso const& b, float t) { vso_lerp(c, out, a, b, t); }

// rasterizer::rasterize_line over the draw's viewport within the render area.
void rasterize_line(rasterizer_state& rs, vso const& v0, vso const& v1) {
  draw_ctx const& c = *rs.c;
  int const nreg = 1 + static_cast<int>(c.nattr);
  vso diff;
  for (auto& r : diff.r) r = mk(0, 0, 0, 0);
  for (int i = 0; i < nreg; ++i) diff.r[i] = sub(v1.r[i], v0.r[i]);
  vec4 const dir = diff.pos();
  float const len_sqr = dir[0] * dir[0] + dir[1] * dir[1];
  vso ddx, ddy;
  float const fx = dir[0] / len_sqr, fy = dir[1] / len_sqr;
  for (int i = 0; i < nreg; ++i) {
    ddx.r[i] = mul(diff.r[i], fx);
    ddy.r[i] = mul(diff.r[i], fy);
  }
  sg_viewport const& vp = c.d->viewport;
  int const left = fast_floori(std::max(0.0f, vp.x)), top = fast_floori(std::max(0.0f, vp.y));
  int const right = fast_floori(std::min(vp.x + vp.w, c.target_w));
  int const bottom = fast_floori(std::min(vp.y + vp.h, c.target_h));
  if (right <= left || bottom <= top) return;
  bool const xmaj = std::fabs(dir[0]) > std::fabs(dir[1]);
  int const ax = xmaj ? 0 : 1, bx = xmaj ? 1 : 0;  // major and minor axis
  float diff_dir = xmaj ? dir[0] : dir[1];
  vso const* start = &v0;
  vso const* end = &v1;
  if (diff_dir < 0) {
    start = &v1;
    end = &v0;
    diff_dir = -diff_dir;
  }
  int const lo = xmaj ? left : top, hi = xmaj ? right : bottom;
  int const mlo = xmaj ? top : left, mhi = xmaj ? bottom : right;
  float const fs = fast_floor(start->pos()[ax] + 0.5f);
  int sx = fast_floori(fs);
  int ex = fast_floori(end->pos()[ax] - 0.5f);
  // clamped to the viewport (rasterize_line clamps the start to hi - 1, which
  // would draw one extrapolated pixel of a line that starts past the right
  // or bottom edge; here such a line draws nothing there)
  sx = std::min(std::max(sx, lo), hi);
  ex = std::min(std::max(ex, lo), hi);
  vec4 more[SG_MAX_COLOR_TARGETS - 1];
  for (int i = sx; i < ex; ++i) {
    float const step = static_cast<float>(i) + 0.5f - start->pos()[ax];
    vso px;
    for (auto& r : px.r) r = mk(0, 0, 0, 0);
    lerp_regs(c, px, *start, *end, step / diff_dir);
    float const m = px.pos()[bx];
    if (m >= static_cast<float>(mhi) || m < static_cast<float>(mlo)) continue;
    int const mi = fast_floori(m);
    if (mi >= mhi) continue;
    // the pixel, and the pixel moved by ddx / ddy, unprojected (the
    // attribute differences are the pixel shader's ddx / ddy)
    vso q[4], sx_, sy_;
    for (int k = 0; k < nreg; ++k) {
      bool const flat = k > 0 && (c.mods[k - 1] & SG_AM_NOINTERPOLATION);  // no derivative
      sx_.r[k] = flat ? px.r[k] : add(px.r[k], ddx.r[k]);
      sy_.r[k] = flat ? px.r[k] : add(px.r[k], ddy.r[k]);
    }
    unproject(c, q[0], px);
    unproject(c, q[1], sx_);
    unproject(c, q[2], sy_);
    q[3] = q[0];
    vec4 out;
    float lod = 0;
    bool have = false;
    bool keep = run_ps(c, q, 0, out, more, lod, have);
    ++rs.st->ps_invocations;
    ++rs.st->backend_input_pixels;
    if (!keep) continue;
    size_t const x = static_cast<size_t>(xmaj ? i : mi), y = static_cast<size_t>(xmaj ? mi : i);
    render_sample(rs, x, y, 0, out, px.pos()[2], true, more);
  }
}

int32_t do_draw(device_state* dev, sg_draw_desc const* d, sg_draw_stats* stats_out) {
  draw_ctx c;
  c.dev = dev;
  c.d = d;
  bool const lines = d->topology == SG_TOPOLOGY_LINE_LIST || d->topology == SG_TOPOLOGY_LINE_STRIP;
  if (!lines && d->topology != SG_TOPOLOGY_TRIANGLE_LIST && d->topology != SG_TOPOLOGY_TRIANGLE_STRIP)
    return SG_INVALID_PARAMETER;
  if (d->raster.fill_mode != SG_FILL_SOLID && d->raster.fill_mode != SG_FILL_WIREFRAME) return SG_INVALID_PARAMETER;
  bool const wire = !lines && d->raster.fill_mode == SG_FILL_WIREFRAME;
  if ((lines || wire) && (d->ps.program >= SG_USER_PROGRAM_BASE || d->bs.program >= SG_USER_PROGRAM_BASE))
    return SG_INVALID_PARAMETER;
  // user programs: registered modules of the stage
  auto user_ok = [&](uint32_t prog, uint32_t stage) {
    if (prog < SG_USER_PROGRAM_BASE) return true;
    size_t const i = prog - SG_USER_PROGRAM_BASE;
    return i < dev->user_shaders.size() && dev->user_shaders[i]->stage == stage;
  };
  if (!user_ok(d->vs.program, SG_STAGE_VERTEX) || !user_ok(d->ps.program, SG_STAGE_PIXEL) ||
      !user_ok(d->bs.program, SG_STAGE_BLEND))
    return SG_INVALID_PARAMETER;
  if (d->num_varyings > SG_MAX_VARYINGS || d->num_inputs > SG_MAX_VS_INPUTS)
    return SG_INVALID_PARAMETER;
  if (d->color_target) {
    auto it = dev->textures.find(d->color_target);
    if (it == dev->textures.end()) return SG_INVALID_PARAMETER;
    c.color = it->second->levels[0].get();
    for (uint32_t i = 0; i + 1 < SG_MAX_COLOR_TARGETS && d->more_color_targets[i]; ++i) {
      auto mt = dev->textures.find(d->more_color_targets[i]);
      if (mt == dev->textures.end()) return SG_INVALID_PARAMETER;
      c.more[c.nmore++] = mt->second->levels[0].get();
    }
  }
  if (d->ds_target) {
    auto it = dev->textures.find(d->ds_target);
    if (it == dev->textures.end()) return SG_INVALID_PARAMETER;
    c.ds = it->second->levels[0].get();
  }
  if (!c.color && !c.ds) return SG_FAILED;
  // set_render_targets (renderer_impl.cpp:159-238)
  c.target_w = c.color ? static_cast<float>(c.color->w) : static_cast<float>(c.ds->w);
  c.target_h = c.color ? static_cast<float>(c.color->h) : static_cast<float>(c.ds->h);
  c.samples = c.color ? c.color->samples : c.ds->samples;
  for (uint32_t i = 0; i < c.nmore; ++i) {  // the smallest colour target; one sample count
    if (c.more[i]->samples != c.samples) return SG_FAILED;
    c.target_w = std::min(c.target_w, static_cast<float>(c.more[i]->w));
    c.target_h = std::min(c.target_h, static_cast<float>(c.more[i]->h));
  }
  if (c.ds && c.color && (c.ds->samples != c.samples || c.ds->w < c.target_w || c.ds->h < c.target_h))
    return SG_FAILED;
  if (c.samples != 1 && c.samples != 2 && c.samples != 4) return SG_INVALID_PARAMETER;
  if (d->vs.samplers[0]) c.vs_samp = &dev->samplers.at(d->vs.samplers[0]);
  if (d->ps.samplers[0]) c.ps_samp = &dev->samplers.at(d->ps.samplers[0]);
  c.nattr = d->num_varyings;
  for (uint32_t i = 0; i < SG_MAX_VARYINGS; ++i) {
    c.mods[i] = d->varying_modifiers[i];
    if (i < c.nattr && (c.mods[i] & SG_AM_CENTROID)) c.has_centroid = true;
  }
  // sample patterns (rasterizer.cpp:1087-1103)
  if (c.samples == 1) {
    c.sp[0][0] = 0.5f; c.sp[0][1] = 0.5f;
  } else if (c.samples == 2) {
    c.sp[0][0] = 0.25f; c.sp[0][1] = 0.25f;
    c.sp[1][0] = 0.75f; c.sp[1][1] = 0.75f;
  } else {
    c.sp[0][0] = 0.375f; c.sp[0][1] = 0.125f;
    c.sp[1][0] = 0.875f; c.sp[1][1] = 0.375f;
    c.sp[2][0] = 0.125f; c.sp[2][1] = 0.625f;
    c.sp[3][0] = 0.625f; c.sp[3][1] = 0.875f;
  }
  c.full_mask = (1ull << c.samples) - 1;
  c.quad_full_mask = c.full_mask | (c.full_mask << 16) | (c.full_mask << 32) | (c.full_mask << 48);
  // early-Z enable (framebuffer.cpp:424); lines test after shading
  c.early_z = c.ds != nullptr && !d->depth_stencil.stencil_enable && !lines && !wire;
  uint32_t const corners = lines ? 2u : 3u;
  c.stats.ia_primitives = d->prim_count;
  c.stats.ia_vertices = uint64_t(corners) * d->prim_count;  // per fetched primitive (default_vertex_cache.cpp:363)
  c.stats.cinvocations = d->prim_count;        // every primitive enters the clipper (geom_setup_engine.cpp:108-123)
  // the GPU path's count (one run per primitive corner); the reference's
  // depends on its worker threads' vertex caches and is not compared
  c.stats.vs_invocations = uint64_t(corners) * d->prim_count;
  if (lines || wire) {
    std::unordered_map<uint32_t, std::unique_ptr<vso>> vcache;
    std::vector<std::unique_ptr<vso>> pool;
    std::vector<vso*> segs;  // pairs, in primitive order
    auto vertex = [&](uint32_t index) {
      auto it = vcache.find(index);
      if (it == vcache.end()) {
        auto v = std::make_unique<vso>();
        for (auto& r : v->r) r = mk(0, 0, 0, 0);
        run_vs(c, index, *v);
        it = vcache.emplace(index, std::move(v)).first;
      }
      return it->second.get();
    };
    for (uint32_t p = 0; p < d->prim_count; ++p) {
      uint32_t idx[3];
      fetch_indexes(c, p, idx);
      if (lines) {
        vso* a = vertex(idx[0]);
        vso* b = vertex(idx[1]);
        if (clip_line(c, a, b, pool)) {
          segs.push_back(a);
          segs.push_back(b);
        }
        continue;
      }
      vso* tv[3] = {vertex(idx[0]), vertex(idx[1]), vertex(idx[2])};
      std::vector<vso*> tri;
      clip_triangle(c, tv, pool, tri);
      for (size_t t = 0; t + 2 < tri.size(); t += 3)
        for (int e = 0; e < 3; ++e) {
          segs.push_back(tri[t + e]);
          segs.push_back(tri[t + (e + 1) % 3]);
        }
    }
    c.stats.cprimitives = segs.size() / 2;
    // project every distinct vertex once, in place
    std::vector<vso*> uniq(segs.begin(), segs.end());
    std::sort(uniq.begin(), uniq.end());
    uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
    for (vso* v : uniq) vp_project(c, *v);
    rasterizer_state rs;
    rs.c = &c;
    rs.tris = nullptr;
    rs.f = ds_functions(c);
    rs.st = &c.stats;
    for (size_t i = 0; i < segs.size(); i += 2) rasterize_line(rs, *segs[i], *segs[i + 1]);
    if (stats_out) *stats_out = c.stats;
    return SG_OK;
  }

  // Vertex processing: the vertex shader is a pure function of the index,
  // so one result per distinct index stands for the reference's caches.
  std::unordered_map<uint32_t, std::unique_ptr<vso>> vcache;
  std::vector<std::unique_ptr<vso>> pool;
  std::vector<vso*> clipped;
  clipped.reserve(size_t(d->prim_count) * 3);
  for (uint32_t p = 0; p < d->prim_count; ++p) {
    uint32_t idx[3];
    fetch_indexes(c, p, idx);
    vso* tv[3];
    for (int i = 0; i < 3; ++i) {
      auto it = vcache.find(idx[i]);
      if (it == vcache.end()) {
        auto v = std::make_unique<vso>();
        for (auto& r : v->r) r = mk(0, 0, 0, 0);
        run_vs(c, idx[i], *v);
        it = vcache.emplace(idx[i], std::move(v)).first;
      }
      tv[i] = it->second.get();
    }
    clip_triangle(c, tv, pool, clipped);
  }
  size_t ntri = clipped.size() / 3;
  c.stats.cprimitives = ntri;
  // viewport_and_project_transform: once per distinct vertex (rasterizer.cpp:1220-1243)
  {
    std::vector<vso*> uniq(clipped.begin(), clipped.end());
    std::sort(uniq.begin(), uniq.end());
    uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
    for (vso* v : uniq) vp_project(c, *v);
  }
  std::vector<tri_info> tris(ntri);
  for (size_t i = 0; i < ntri; ++i) {
    vso const* vv[3] = {clipped[i * 3 + 0], clipped[i * 3 + 1], clipped[i * 3 + 2]};
    compute_tri(c, vv, tris[i]);
  }
  // tile binning (rasterizer.cpp:775-862); lists come out in primitive order
  int tx_n = static_cast<int>(static_cast<size_t>(d->viewport.w + TILE - 1) / TILE);
  int ty_n = static_cast<int>(static_cast<size_t>(d->viewport.h + TILE - 1) / TILE);
  std::vector<std::vector<uint32_t>> bins(size_t(tx_n) * ty_n);
  for (size_t i = 0; i < ntri; ++i) {
    tri_info const& ti = tris[i];
    if (!ti.v0) continue;
    int sx = std::min(fast_floori(std::max(0.0f, ti.bbox[0]) / TILE), tx_n);
    int sy = std::min(fast_floori(std::max(0.0f, ti.bbox[2]) / TILE), ty_n);
    int ex = std::min(fast_ceili(std::max(0.0f, ti.bbox[1]) / TILE) + 1, tx_n);
    int ey = std::min(fast_ceili(std::max(0.0f, ti.bbox[3]) / TILE) + 1, ty_n);
    uint32_t id = static_cast<uint32_t>(i);
    if (sx + 1 == ex && sy + 1 == ey) {
      bins[size_t(sy) * tx_n + sx].push_back(id << 1);
      continue;
    }
    bool mx[3], my[3];
    float stx[3], sty[3], r2a[3];
    for (int e = 0; e < 3; ++e) {
      mx[e] = ti.edge[e][0] > 0;
      my[e] = ti.edge[e][1] > 0;
      stx[e] = TILE * ti.edge[e][0];
      sty[e] = TILE * ti.edge[e][1];
      r2a[e] = -std::fabs(stx[e]) - std::fabs(sty[e]);
    }
    for (int y = sy; y < ey; ++y)
      for (int x = sx; x < ex; ++x) {
        int rej = 0, acc = 1;
        for (int e = 0; e < 3; ++e) {
          float evv = ti.edge[e][2] - (static_cast<float>(x + mx[e]) * TILE * ti.edge[e][0] +
                                       static_cast<float>(y + my[e]) * TILE * ti.edge[e][1]);
          rej |= (0 < evv);
          acc &= (r2a[e] >= evv);
        }
        if (!rej) bins[size_t(y) * tx_n + x].push_back((id << 1) | static_cast<uint32_t>(acc));
      }
  }
  rasterizer_state rs;
  rs.c = &c;
  rs.tris = &tris;
  rs.f = ds_functions(c);
  rs.st = &c.stats;
  for (int ty = 0; ty < ty_n; ++ty)
    for (int tx = 0; tx < tx_n; ++tx) {
      auto const& list = bins[size_t(ty) * tx_n + tx];
      for (uint32_t e : list)
        rasterize_triangle(rs, e, static_cast<float>(tx * TILE), static_cast<float>(ty * TILE));
    }
  if (stats_out) *stats_out = c.stats;
  return SG_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
struct sg_device {
  device_state st;
};

extern "C" {

int32_t sg_device_create(int32_t, void*, sg_device** out) {
  *out = new sg_device();
  return SG_OK;
}
void sg_device_destroy(sg_device* d) { delete d; }
int32_t sg_sync(sg_device*) { return SG_OK; }
const char* sg_last_error(sg_device*) { return ""; }
// The restatement is synchronous and keeps no stage timers.
int32_t sg_profile_enable(sg_device*, int32_t) { return SG_OK; }
int32_t sg_profile_read(sg_device*, sg_profile_data* out) {
  if (!out) return SG_INVALID_PARAMETER;
  std::memset(out, 0, sizeof(*out));
  return SG_OK;
}

int32_t sg_buffer_create(sg_device* d, size_t size, uint32_t* out) {
  *out = d->st.next++;
  d->st.buffers[*out].assign(size, 0);
  return SG_OK;
}
int32_t sg_buffer_upload(sg_device* d, uint32_t b, size_t off, const void* src, size_t size) {
  auto it = d->st.buffers.find(b);
  if (it == d->st.buffers.end() || off + size > it->second.size()) return SG_INVALID_PARAMETER;
  std::memcpy(it->second.data() + off, src, size);
  return SG_OK;
}
int32_t sg_buffer_download(sg_device* d, uint32_t b, size_t off, void* dst, size_t size) {
  auto it = d->st.buffers.find(b);
  if (it == d->st.buffers.end() || off + size > it->second.size()) return SG_INVALID_PARAMETER;
  std::memcpy(dst, it->second.data() + off, size);
  return SG_OK;
}
int32_t sg_buffer_destroy(sg_device* d, uint32_t b) {
  d->st.buffers.erase(b);
  return SG_OK;
}

int32_t sg_texture_create(sg_device* d, uint32_t w, uint32_t h, uint32_t s, uint32_t fmt,
                          uint32_t* out) {
  if (elem_size(fmt) == 0 || w == 0 || h == 0 || w > SG_MAX_RT_SIZE || h > SG_MAX_RT_SIZE)
    return SG_INVALID_PARAMETER;
  if (s != 1 && s != 2 && s != 4) return SG_INVALID_PARAMETER;
  auto t = std::make_unique<texture>();
  t->width = w;
  t->height = h;
  t->levels.push_back(std::make_unique<surface>(w, h, s, fmt));
  *out = d->st.next++;
  d->st.textures[*out] = std::move(t);
  return SG_OK;
}
// renderer::create_texcube: six faces (texture_cube.cpp:12-16)
int32_t sg_texture_create_cube(sg_device* d, uint32_t w, uint32_t h, uint32_t s, uint32_t fmt, uint32_t* out) {
  int32_t r = sg_texture_create(d, w, h, s, fmt, out);
  if (r != SG_OK) return r;
  texture& t = *d->st.textures[*out];
  t.cube = true;
  for (int f = 1; f < 6; ++f) t.levels.push_back(std::make_unique<surface>(w, h, s, fmt));
  return SG_OK;
}
static surface* level_of(sg_device* d, uint32_t t, uint32_t level) {
  auto it = d->st.textures.find(t);
  if (it == d->st.textures.end() || level >= it->second->levels.size()) return nullptr;
  return it->second->levels[level].get();
}
int32_t sg_texture_upload(sg_device* d, uint32_t t, uint32_t level, const void* src, size_t size) {
  surface* s = level_of(d, t, level);
  if (!s || size != s->data.size()) return SG_INVALID_PARAMETER;
  std::memcpy(s->data.data(), src, size);
  return SG_OK;
}
int32_t sg_texture_download(sg_device* d, uint32_t t, uint32_t level, void* dst, size_t size) {
  surface* s = level_of(d, t, level);
  if (!s || size != s->data.size()) return SG_INVALID_PARAMETER;
  std::memcpy(dst, s->data.data(), size);
  return SG_OK;
}
int32_t sg_texture_gen_mipmap(sg_device* d, uint32_t t, uint32_t filter) {
  auto it = d->st.textures.find(t);
  if (it == d->st.textures.end()) return SG_INVALID_PARAMETER;
  texture& tx = *it->second;
  if (tx.cube) return SG_INVALID_PARAMETER;  // texture_cube::gen_mipmap reads a size it never set
  uint32_t nlev = lod_limit(tx.width, tx.height);
  tx.levels.resize(1);
  for (uint32_t l = 1; l < nlev; ++l) tx.levels.push_back(make_mip(*tx.levels.back(), filter));
  return SG_OK;
}
int32_t sg_texture_info(sg_device* d, uint32_t t, uint32_t level, uint32_t* w, uint32_t* h,
                        uint32_t* s, uint32_t* fmt, uint32_t* levels) {
  surface* sf = level_of(d, t, level);
  if (!sf) return SG_INVALID_PARAMETER;
  if (w) *w = sf->w;
  if (h) *h = sf->h;
  if (s) *s = sf->samples;
  if (fmt) *fmt = sf->fmt;
  if (levels) *levels = static_cast<uint32_t>(d->st.textures[t]->levels.size());
  return SG_OK;
}
int32_t sg_texture_destroy(sg_device* d, uint32_t t) {
  d->st.textures.erase(t);
  return SG_OK;
}
int32_t sg_sampler_create(sg_device* d, const sg_sampler_desc* desc, uint32_t tex, uint32_t* out) {
  auto it = d->st.textures.find(tex);
  if (it == d->st.textures.end()) return SG_INVALID_PARAMETER;
  sampler s;
  s.d = *desc;
  s.tex = it->second.get();
  *out = d->st.next++;
  d->st.samplers[*out] = s;
  return SG_OK;
}
int32_t sg_sampler_destroy(sg_device* d, uint32_t s) {
  d->st.samplers.erase(s);
  return SG_OK;
}
int32_t sg_draw(sg_device* d, const sg_draw_desc* desc, sg_draw_stats* stats) {
  if (!d || !desc) return SG_INVALID_PARAMETER;
  return do_draw(&d->st, desc, stats);
}
// surface::fill (surface.cpp:170-275) via render_core::clear_color
int32_t sg_clear_color(sg_device* d, uint32_t t, const float rgba[4]) {
  surface* s = level_of(d, t, 0);
  if (!s) return SG_INVALID_PARAMETER;
  std::vector<uint8_t> px(s->esz);
  write_texel(s->fmt, px.data(), mk(rgba[0], rgba[1], rgba[2], rgba[3]));
  for (size_t i = 0; i < s->data.size(); i += s->esz) std::memcpy(&s->data[i], px.data(), s->esz);
  return SG_OK;
}
// render_core::clear_depth_stencil / framebuffer::clear_depth_stencil
// (render_core.cpp:100-111, framebuffer.cpp:616-644)
int32_t sg_clear_depth_stencil(sg_device* d, uint32_t t, uint32_t flags, float depth,
                               uint32_t stencil) {
  surface* s = level_of(d, t, 0);
  if (!s) return SG_INVALID_PARAMETER;
  if (flags == 0 || flags > 3) return SG_INVALID_PARAMETER;
  for (size_t i = 0; i < s->data.size(); i += s->esz) {
    uint8_t* p = &s->data[i];
    switch (s->fmt) {
    case SG_FMT_RG32F:
      if (flags & SG_CLEAR_DEPTH) std::memcpy(p, &depth, 4);
      if (flags & SG_CLEAR_STENCIL) std::memcpy(p + 4, &stencil, 4);
      break;
    case SG_FMT_D32F:
      if (flags & SG_CLEAR_DEPTH) std::memcpy(p, &depth, 4);
      break;
    case SG_FMT_D24S8: {
      uint32_t w;
      std::memcpy(&w, p, 4);
      if (flags & SG_CLEAR_DEPTH) w = (w & 0xFF000000u) | d24_quantize(depth);
      if (flags & SG_CLEAR_STENCIL) w = (w & 0x00FFFFFFu) | ((stencil & 0xFFu) << 24);
      std::memcpy(p, &w, 4);
      break;
    }
    default: return SG_INVALID_PARAMETER;
    }
  }
  return SG_OK;
}
// surface::resolve (surface.cpp:123-140)
int32_t sg_resolve(sg_device* d, uint32_t src, uint32_t dst) {
  surface* a = level_of(d, src, 0);
  surface* b = level_of(d, dst, 0);
  if (!a || !b || b->samples != 1 || a->w != b->w || a->h != b->h) return SG_INVALID_PARAMETER;
  float inv = 1 / static_cast<float>(a->samples);
  for (uint32_t y = 0; y < a->h; ++y)
    for (uint32_t x = 0; x < a->w; ++x) {
      vec4 c = mk(0, 0, 0, 0);
      for (uint32_t s = 0; s < a->samples; ++s) c = add(c, a->get(x, y, s));
      b->set(x, y, 0, mul(c, inv));
    }
  return SG_OK;
}

int32_t sg_shader_register(sg_device* d, const sg_shader_module* m, uint32_t* out) {
  if (!d || !m || !out || m->abi_version != SG_SHADER_ABI_VERSION ||
      (m->stage == SG_STAGE_PIXEL && !m->host_ps) || (m->stage == SG_STAGE_BLEND && !m->host_bs) ||
      (m->stage == SG_STAGE_VERTEX && !m->host_vs) ||
      (m->stage != SG_STAGE_PIXEL && m->stage != SG_STAGE_BLEND && m->stage != SG_STAGE_VERTEX))
    return SG_INVALID_PARAMETER;
  auto& v = d->st.user_shaders;
  for (size_t i = 0; i < v.size(); ++i)
    if (v[i] == m) {
      *out = SG_USER_PROGRAM_BASE + static_cast<uint32_t>(i);
      return SG_OK;
    }
  v.push_back(m);
  *out = SG_USER_PROGRAM_BASE + static_cast<uint32_t>(v.size() - 1);
  return SG_OK;
}

// The command list of sg_submit, executed one command at a time
// (render_core::execute in order, render_core.cpp:30-61).
int32_t sg_submit(sg_device* d, const sg_command* cmds, uint32_t n, sg_draw_stats* stats) {
  if (!d || (!cmds && n)) return SG_INVALID_PARAMETER;
  if (stats) std::memset(stats, 0, sizeof(sg_draw_stats) * n);
  for (uint32_t i = 0; i < n; ++i) {
    sg_command const& c = cmds[i];
    int32_t r;
    switch (c.type) {
    case SG_CMD_DRAW: r = sg_draw(d, c.draw, stats ? &stats[i] : nullptr); break;
    case SG_CMD_CLEAR_COLOR: r = sg_clear_color(d, c.texture, c.color); break;
    case SG_CMD_CLEAR_DEPTH_STENCIL: r = sg_clear_depth_stencil(d, c.texture, c.flags, c.depth, c.stencil); break;
    case SG_CMD_RESOLVE: r = sg_resolve(d, c.texture, c.texture2); break;
    default: r = SG_INVALID_PARAMETER; break;
    }
    if (r != SG_OK) return r;
  }
  return SG_OK;
}

}  // extern "C"
