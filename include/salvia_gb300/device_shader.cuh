// salvia_gb300/device_shader.cuh -- user shader bodies for the GB300 pipeline.
//
// The reference's applications write shaders as C++ classes deriving from
// cpp_vertex_shader / cpp_pixel_shader / cpp_blend_shader and overriding
// shader_prog (salvia/include/salvia/core/shader.h:159-215).  Here such a
// class derives from salvia_gb300::vertex_shader, pixel_shader or
// blend_shader, with the same shader_prog signatures and the same helpers
// (ddx, ddy, tex2d, tex2dlod, tex2dproj, front_face; pixel_accessor::color;
// a vertex shader's sampler lookup), written __host__ __device__, and is
// exported as a shader module:
//
//     #include <salvia_gb300/device_shader.cuh>
//     struct my_ps : salvia_gb300::pixel_shader {
//       __host__ __device__ bool shader_prog(salvia_gb300::vs_output const& in,
//                                            salvia_gb300::ps_output& out) const {
//         out.color[0] = tex2d(0) * in.attribute(1);
//         return out.color[0].w >= constant(0);   // false discards
//       }
//     };
//     SALVIA_GB300_PIXEL_SHADER(my_ps)   // extern "C" salvia_gb300_module_my_ps()
//
//     struct my_vs : salvia_gb300::vertex_shader {
//       __host__ __device__ void shader_prog(salvia_gb300::vs_input const& in,
//                                            salvia_gb300::vs_output& out) const {
//         out.position = in.attribute(0) * constant(0);
//         out.attribute(0) = in.attribute(1);
//       }
//     };
//     SALVIA_GB300_VERTEX_SHADER(my_vs)
//
// compiled with nvcc for sm_103a into the application (or a shared object):
//
//     nvcc -gencode arch=compute_103a,code=sm_103a -fmad=false -std=c++17 \
//          -I<repo>/include -I<repo>/salviarenderer_gb300/csrc ...
//
// (-fmad=false keeps the interpolation's float operations as the reference
// orders them).  sg_shader_register(dev, salvia_gb300_module_my_ps(), &id)
// then makes `id` a program for sg_shader.program.  The module holds the
// pass kernels instantiated for the class -- the pixel-shading kernel or the
// output merger -- in the application's own code, and the body compiled for
// the host, which CPU backends of the same C ABI run.
//
// Pixel-shader helpers read sampler slot 0 and the pixel shader's constants.
// tex2d, tex2dlod and sample are lookups without anisotropy parameters: on an
// anisotropic sampler (mip filter anisotropic) the reference dereferences
// the absent parameters (sampler.cpp:730-755), so a body uses sample_grad
// (sampler::sample_2d_grad) there;
// ddx / ddy are the differences of the quad's pixels (cpp_pixel_shader.cpp:
// 13-19) and may be called anywhere in the body.  On the host the helpers
// are the backend's own (sg_host_ps_io), so a CPU backend -- the reference
// renderer itself -- runs the same body with its own tex2d and derivatives.
#pragma once

#include <cstdint>

#include "salvia_gb300.h"

#ifdef __CUDACC__
#include "sg_geometry.cuh"
#include "sg_raster.cuh"
#else
// a host compiler builds the bodies for CPU backends only
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#endif

namespace salvia_gb300 {

struct vec4 {
  float x = 0.0f, y = 0.0f, z = 0.0f, w = 0.0f;
  __host__ __device__ vec4() {}
  __host__ __device__ vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
  __host__ __device__ float operator[](int i) const { return i == 0 ? x : i == 1 ? y : i == 2 ? z : w; }
};
__host__ __device__ inline vec4 operator+(vec4 a, vec4 b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__host__ __device__ inline vec4 operator-(vec4 a, vec4 b) { return vec4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
__host__ __device__ inline vec4 operator*(vec4 a, vec4 b) { return vec4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
__host__ __device__ inline vec4 operator*(vec4 a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }
__host__ __device__ inline vec4 operator/(vec4 a, float s) { return vec4(a.x / s, a.y / s, a.z / s, a.w / s); }
__host__ __device__ inline vec4 lerp(vec4 a, vec4 b, float t) {  // a + (b - a) * t, per component
  return vec4(a.x + (b.x - a.x) * t, a.y + (b.y - a.y) * t, a.z + (b.z - a.z) * t, a.w + (b.w - a.w) * t);
}

// shader_regs.h:32-113: the pixel's interpolated position and varyings, and
// the colours a pixel shader writes (one per colour target).
struct vs_output {
  vec4 position;
  vec4 attr[SG_MAX_VARYINGS];
  __host__ __device__ vec4 const& attribute(int i) const { return attr[i]; }
  __host__ __device__ vec4& attribute(int i) { return attr[i]; }
};
// shader_regs.h:16-30: a vertex's input registers (the draw's inputs in order)
struct vs_input {
  vec4 attr[SG_MAX_VS_INPUTS];
  __host__ __device__ vec4 const& attribute(int i) const { return attr[i]; }
};
struct ps_output {
  vec4 color[SG_MAX_COLOR_TARGETS];
};

namespace detail {
// The device-side context of one pixel of a quad, set by the kernel.
struct ps_device_ctx;
// Gives a shader body's base class its context (device kernel or host io).
struct shader_access;
}  // namespace detail

// Base of a user vertex shader (cpp_vertex_shader, shader.h:159-165).  The
// number and modifiers of its outputs are the draw's num_varyings and
// varying_modifiers.
class vertex_shader {
  friend struct detail::shader_access;
  void const* ctx_ = nullptr;  // DrawParams (device) or sg_host_vs_io (host)

protected:
  // sampler::sample(u, v, lod) on sampler slot 0 of the vertex shader
  // (vertex texture fetch)
  __host__ __device__ vec4 sample(float u, float v, float lod) const;
  __host__ __device__ float constant(int i) const;
};

// Base of a user pixel shader (cpp_pixel_shader, shader.h:169-205).
class pixel_shader {
  friend struct detail::shader_access;
  void const* ctx_ = nullptr;  // ps_device_ctx (device) or sg_host_ps_io (host)

protected:
  __host__ __device__ vec4 ddx(int reg) const;
  __host__ __device__ vec4 ddy(int reg) const;
  // tex2d(sampler, reg): the level from the quad differences of the register
  // (cpp_pixel_shader.cpp:23-31)
  __host__ __device__ vec4 tex2d(int reg) const;
  // tex2dlod(sampler, reg): the register's w is the level (cpp_pixel_shader.cpp:33-40)
  __host__ __device__ vec4 tex2dlod(int reg) const;
  // tex2dproj(sampler, reg) (cpp_pixel_shader.cpp:42-60)
  __host__ __device__ vec4 tex2dproj(int reg) const;
  // sampler::sample(u, v, lod) and sample_2d_grad
  __host__ __device__ vec4 sample(float u, float v, float lod) const;
  __host__ __device__ vec4 sample_grad(float u, float v, float dxu, float dxv, float dyu, float dyv) const;
  // sampler::sample_cube(x, y, z, lod) (sampler.cpp:771-829)
  __host__ __device__ vec4 sample_cube(float x, float y, float z, float lod) const;
  __host__ __device__ bool front_face() const;
  __host__ __device__ float constant(int i) const;
};

// pixel_accessor (pixel_accessor.h): the colour targets at one pixel.
class pixel_accessor {
  friend struct detail::shader_access;
  void const* ctx_ = nullptr;
  uint32_t x_ = 0, y_ = 0;

public:
  __host__ __device__ vec4 color(int target, int sample) const;
  __host__ __device__ void color(int target, int sample, vec4 const& c) const;
};

// Base of a user blend shader (cpp_blend_shader, shader.h:209-215).
class blend_shader {
  friend struct detail::shader_access;
  void const* ctx_ = nullptr;  // DrawParams (device) or sg_host_bs_io (host)

protected:
  __host__ __device__ float constant(int i) const;
};

// ---------------------------------------------------------------------------
// implementation

namespace detail {

#ifdef __CUDACC__
// One pixel of a quad of a fragment: the triangle, the draw, the pixel's
// interpolation offsets and 1/w (k_shade's, pixel by pixel).
struct ps_device_ctx {
  sg::TriView t;
  sg::DrawParams const* D;
  float dx, dy;        // the quad's offsets from v0
  float pdx[4], pdy[4];  // centroid-adjusted offsets of each pixel (centroid draws)
  float invw[4];
  bool centroid;
  bool front;
  int pixel;
};

// element p of a quad's four values, selected rather than indexed (the
// context stays in registers)
__device__ __forceinline__ float quad_sel(float const (&a)[4], int p) {
  return p == 0 ? a[0] : p == 1 ? a[1] : p == 2 ? a[2] : a[3];
}

// Register `reg` (0-based varying) of `pixel` exactly as k_shade computes it
// (step_2d_unproj_attr_n_quad / step_2d_unproj_attr_n, shader.cpp:208-367).
__device__ inline sg::v4 pixel_attr(ps_device_ctx const& c, int reg, int p) {
  using namespace sg;
  if (reg < 0 || static_cast<uint32_t>(reg) >= c.D->nattr) return mk4(0, 0, 0, 0);
  v4 in = c.t.v0(1 + reg), d0 = c.t.ddx(1 + reg), d1 = c.t.ddy(1 + reg);
  uint32_t const mods = c.D->mods[reg];
  v4 a;
  if (mods & SG_AM_NOINTERPOLATION) {
    a = in;
  } else if (c.centroid) {
    float const px = quad_sel(c.pdx, p), py = quad_sel(c.pdy, p);
    a = mk4(in.x + (d0.x * px + d1.x * py), in.y + (d0.y * px + d1.y * py), in.z + (d0.z * px + d1.z * py),
            in.w + (d0.w * px + d1.w * py));
  } else {
    v4 a00 = mk4(in.x + (d0.x * c.dx + d1.x * c.dy), in.y + (d0.y * c.dx + d1.y * c.dy),
                 in.z + (d0.z * c.dx + d1.z * c.dy), in.w + (d0.w * c.dx + d1.w * c.dy));
    a = p == 0 ? a00 : p == 1 ? a00 + d0 : p == 2 ? a00 + d1 : (a00 + d0) + d1;
  }
  return (mods & SG_AM_NOPERSPECTIVE) ? a : a * quad_sel(c.invw, p);
}
__device__ inline vec4 to_vec4(sg::v4 v) { return vec4(v.x, v.y, v.z, v.w); }
#endif

struct shader_access {
  __host__ __device__ static void bind(vertex_shader& s, void const* ctx) { s.ctx_ = ctx; }
  __host__ __device__ static void bind(pixel_shader& s, void const* ctx) { s.ctx_ = ctx; }
  __host__ __device__ static void bind(blend_shader& s, void const* ctx) { s.ctx_ = ctx; }
  __host__ __device__ static void bind(pixel_accessor& a, void const* ctx, uint32_t x, uint32_t y) {
    a.ctx_ = ctx;
    a.x_ = x;
    a.y_ = y;
  }
};

inline vec4 host_out(float const* o) { return vec4(o[0], o[1], o[2], o[3]); }
// a backend helper of the host io on register `reg`
inline vec4 host_call(sg_host_ps_io const* io, void (*fn)(void*, uint32_t, float*), int reg) {
  float o[4] = {0, 0, 0, 0};
  if (reg >= 0 && reg < SG_MAX_VARYINGS) fn(io->backend, static_cast<uint32_t>(reg), o);
  return host_out(o);
}

}  // namespace detail

// (device helpers: a draw without a sampler in the slot samples zeros)
__host__ __device__ inline vec4 vertex_shader::sample(float u, float v, float lod) const {
#ifdef __CUDA_ARCH__
  sg::dev_sampler const& sp = static_cast<sg::DrawParams const*>(ctx_)->vs_samp;
  if (sp.nlevels <= 0) return vec4();
  return detail::to_vec4(sg::sample_impl(sp, u, v, lod, nullptr));
#else
  auto io = static_cast<sg_host_vs_io const*>(ctx_);
  float o[4] = {0, 0, 0, 0};
  io->sample(io->backend, u, v, lod, o);
  return detail::host_out(o);
#endif
}
__host__ __device__ inline float vertex_shader::constant(int i) const {
  if (i < 0 || i >= SG_MAX_SHADER_CONSTANTS) return 0.0f;
#ifdef __CUDA_ARCH__
  return static_cast<sg::DrawParams const*>(ctx_)->vs_k[i];
#else
  return static_cast<sg_host_vs_io const*>(ctx_)->constants[i];
#endif
}

#ifdef __CUDA_ARCH__
#define SALVIA_GB300_PS_CTX (*static_cast<detail::ps_device_ctx const*>(ctx_))
#endif

__host__ __device__ inline vec4 pixel_shader::ddx(int reg) const {
#ifdef __CUDA_ARCH__
  return detail::to_vec4(detail::pixel_attr(SALVIA_GB300_PS_CTX, reg, 1) - detail::pixel_attr(SALVIA_GB300_PS_CTX, reg, 0));
#else
  auto io = static_cast<sg_host_ps_io const*>(ctx_);
  return detail::host_call(io, io->ddx, reg);
#endif
}
__host__ __device__ inline vec4 pixel_shader::ddy(int reg) const {
#ifdef __CUDA_ARCH__
  return detail::to_vec4(detail::pixel_attr(SALVIA_GB300_PS_CTX, reg, 2) - detail::pixel_attr(SALVIA_GB300_PS_CTX, reg, 0));
#else
  auto io = static_cast<sg_host_ps_io const*>(ctx_);
  return detail::host_call(io, io->ddy, reg);
#endif
}
__host__ __device__ inline vec4 pixel_shader::sample(float u, float v, float lod) const {
#ifdef __CUDA_ARCH__
  if (SALVIA_GB300_PS_CTX.D->ps_samp.nlevels <= 0) return vec4();
  return detail::to_vec4(sg::sample_impl(SALVIA_GB300_PS_CTX.D->ps_samp, u, v, lod, nullptr));
#else
  auto io = static_cast<sg_host_ps_io const*>(ctx_);
  float o[4];
  io->sample(io->backend, u, v, lod, o);
  return detail::host_out(o);
#endif
}
__host__ __device__ inline vec4 pixel_shader::sample_grad(float u, float v, float dxu, float dxv, float dyu,
                                                          float dyv) const {
#ifdef __CUDA_ARCH__
  if (SALVIA_GB300_PS_CTX.D->ps_samp.nlevels <= 0) return vec4();
  return detail::to_vec4(sg::sample_2d_grad(SALVIA_GB300_PS_CTX.D->ps_samp, u, v, dxu, dxv, dyu, dyv, 0.0f));
#else
  auto io = static_cast<sg_host_ps_io const*>(ctx_);
  float o[4];
  io->sample_grad(io->backend, u, v, dxu, dxv, dyu, dyv, o);
  return detail::host_out(o);
#endif
}
__host__ __device__ inline vec4 pixel_shader::sample_cube(float x, float y, float z, float lod) const {
#ifdef __CUDA_ARCH__
  if (SALVIA_GB300_PS_CTX.D->ps_samp.nlevels <= 0) return vec4();
  return detail::to_vec4(sg::sample_cube(SALVIA_GB300_PS_CTX.D->ps_samp, x, y, z, lod));
#else
  auto io = static_cast<sg_host_ps_io const*>(ctx_);
  float o[4];
  io->sample_cube(io->backend, x, y, z, lod, o);
  return detail::host_out(o);
#endif
}
__host__ __device__ inline vec4 pixel_shader::tex2d(int reg) const {
#ifdef __CUDA_ARCH__
  vec4 const dx = ddx(reg), dy = ddy(reg);
  detail::ps_device_ctx const& c = SALVIA_GB300_PS_CTX;
  sg::v4 const a = detail::pixel_attr(c, reg, c.pixel);
  float const lod = sg::calc_lod_2d(c.D->ps_samp, dx.x, dx.y, dy.x, dy.y);
  return sample(a.x, a.y, lod);
#else
  auto io = static_cast<sg_host_ps_io const*>(ctx_);
  return detail::host_call(io, io->tex2d, reg);
#endif
}
__host__ __device__ inline vec4 pixel_shader::tex2dlod(int reg) const {
#ifdef __CUDA_ARCH__
  detail::ps_device_ctx const& c = SALVIA_GB300_PS_CTX;
  sg::v4 const a = detail::pixel_attr(c, reg, c.pixel);
  return sample(a.x, a.y, a.w);
#else
  auto io = static_cast<sg_host_ps_io const*>(ctx_);
  return detail::host_call(io, io->tex2dlod, reg);
#endif
}
__host__ __device__ inline vec4 pixel_shader::tex2dproj(int reg) const {
#ifdef __CUDA_ARCH__
  vec4 const a = detail::to_vec4(detail::pixel_attr(SALVIA_GB300_PS_CTX, reg, SALVIA_GB300_PS_CTX.pixel));
  vec4 const nx = a + ddx(reg), ny = a + ddy(reg);
  float const px = (a.x / a.w + 1.0f) * 0.5f, py = (a.y / a.w + 1.0f) * 0.5f;
  float const qxx = (nx.x / nx.w + 1.0f) * 0.5f, qxy = (nx.y / nx.w + 1.0f) * 0.5f;
  float const qyx = (ny.x / ny.w + 1.0f) * 0.5f, qyy = (ny.y / ny.w + 1.0f) * 0.5f;
  return sample_grad(px, py, qxx - px, qxy - py, qyx - px, qyy - py);
#else
  auto io = static_cast<sg_host_ps_io const*>(ctx_);
  return detail::host_call(io, io->tex2dproj, reg);
#endif
}
__host__ __device__ inline bool pixel_shader::front_face() const {
#ifdef __CUDA_ARCH__
  return SALVIA_GB300_PS_CTX.front;
#else
  return static_cast<sg_host_ps_io const*>(ctx_)->front_face != 0;
#endif
}
__host__ __device__ inline float pixel_shader::constant(int i) const {
  if (i < 0 || i >= SG_MAX_SHADER_CONSTANTS) return 0.0f;
#ifdef __CUDA_ARCH__
  return SALVIA_GB300_PS_CTX.D->ps_k[i];
#else
  return static_cast<sg_host_ps_io const*>(ctx_)->constants[i];
#endif
}

__host__ __device__ inline float blend_shader::constant(int i) const {
  if (i < 0 || i >= SG_MAX_SHADER_CONSTANTS) return 0.0f;
#ifdef __CUDA_ARCH__
  return static_cast<sg::DrawParams const*>(ctx_)->bs_k[i];
#else
  return static_cast<sg_host_bs_io const*>(ctx_)->constants[i];
#endif
}

__host__ __device__ inline vec4 pixel_accessor::color(int target, int sample) const {
#ifdef __CUDA_ARCH__
  sg::TargetParams const& T = *static_cast<sg::TargetParams const*>(ctx_);
  if (target == 0 && T.color)
    return detail::to_vec4(sg::read_texel(T.color_fmt, sg::color_addr(T, x_, y_, sample)));
  if (target > 0 && static_cast<uint32_t>(target) <= T.nmore) {
    int const i = target - 1;
    return detail::to_vec4(sg::read_texel(
        T.more_fmt[i],
        T.more_color[i] + ((static_cast<size_t>(y_) * T.more_stride[i] + x_) * T.samples + sample) * T.more_esz[i]));
  }
  return vec4();
#else
  auto io = static_cast<sg_host_bs_io const*>(ctx_);
  float o[4] = {0, 0, 0, 0};
  io->get(io->backend, static_cast<uint32_t>(target), static_cast<uint32_t>(sample), o);
  return detail::host_out(o);
#endif
}
__host__ __device__ inline void pixel_accessor::color(int target, int sample, vec4 const& c) const {
#ifdef __CUDA_ARCH__
  sg::TargetParams const& T = *static_cast<sg::TargetParams const*>(ctx_);
  sg::v4 const v = sg::mk4(c.x, c.y, c.z, c.w);
  if (target == 0 && T.color) {
    sg::write_texel(T.color_fmt, sg::color_addr(T, x_, y_, sample), v);
  } else if (target > 0 && static_cast<uint32_t>(target) <= T.nmore) {
    int const i = target - 1;
    sg::write_texel(T.more_fmt[i],
                    T.more_color[i] +
                        ((static_cast<size_t>(y_) * T.more_stride[i] + x_) * T.samples + sample) * T.more_esz[i],
                    v);
  }
#else
  auto io = static_cast<sg_host_bs_io const*>(ctx_);
  float const o[4] = {c.x, c.y, c.z, c.w};
  io->set(io->backend, static_cast<uint32_t>(target), static_cast<uint32_t>(sample), o);
#endif
}

}  // namespace salvia_gb300

// The body compiled for the host: the sg_host_*_io entry of a module.
#define SALVIA_GB300_HOST_VE_(cls)                                                                  \
  static int32_t salvia_gb300_host_##cls(sg_host_vs_io* io) {                                                \
    salvia_gb300::vs_input in;                                                                                 \
    for (int i = 0; i < SG_MAX_VS_INPUTS; ++i) in.attr[i] = salvia_gb300::detail::host_out(io->in[i]);        \
    salvia_gb300::vs_output out;                                                                               \
    cls vs;                                                                                                    \
    salvia_gb300::detail::shader_access::bind(vs, io);                                                         \
    vs.shader_prog(in, out);                                                                                   \
    io->position[0] = out.position.x;                                                                          \
    io->position[1] = out.position.y;                                                                          \
    io->position[2] = out.position.z;                                                                          \
    io->position[3] = out.position.w;                                                                          \
    for (int i = 0; i < SG_MAX_VARYINGS; ++i) {                                                                \
      io->attr[i][0] = out.attr[i].x;                                                                          \
      io->attr[i][1] = out.attr[i].y;                                                                          \
      io->attr[i][2] = out.attr[i].z;                                                                          \
      io->attr[i][3] = out.attr[i].w;                                                                          \
    }                                                                                                          \
    return 1;                                                                                                  \
  }

#define SALVIA_GB300_HOST_PI_(cls)                                                                  \
  static int32_t salvia_gb300_host_##cls(sg_host_ps_io* io) {                                                \
    salvia_gb300::vs_output in;                                                                                \
    float const* p = io->position;                                                                             \
    in.position = salvia_gb300::vec4(p[0], p[1], p[2], p[3]);                                                  \
    for (int i = 0; i < SG_MAX_VARYINGS; ++i) in.attr[i] = salvia_gb300::detail::host_out(io->attr[i]);      \
    salvia_gb300::ps_output out;                                                                               \
    cls ps;                                                                                                    \
    salvia_gb300::detail::shader_access::bind(ps, io);                                                         \
    bool const keep = ps.shader_prog(in, out);                                                                 \
    for (int i = 0; i < SG_MAX_COLOR_TARGETS; ++i) {                                                           \
      io->color[i][0] = out.color[i].x;                                                                        \
      io->color[i][1] = out.color[i].y;                                                                        \
      io->color[i][2] = out.color[i].z;                                                                        \
      io->color[i][3] = out.color[i].w;                                                                        \
    }                                                                                                          \
    return keep ? 1 : 0;                                                                                       \
  }

#define SALVIA_GB300_HOST_BL_(cls)                                                                  \
  static int32_t salvia_gb300_host_##cls(sg_host_bs_io* io) {                                                \
    salvia_gb300::ps_output in;                                                                                \
    for (int i = 0; i < SG_MAX_COLOR_TARGETS; ++i) in.color[i] = salvia_gb300::detail::host_out(io->in_color[i]); \
    cls bs;                                                                                                    \
    salvia_gb300::detail::shader_access::bind(bs, io);                                                         \
    salvia_gb300::pixel_accessor acc;                                                                          \
    salvia_gb300::detail::shader_access::bind(acc, io, 0u, 0u);                                                \
    return bs.shader_prog(io->sample, acc, in) ? 1 : 0;                                                        \
  }

// ---------------------------------------------------------------------------
// the kernels instantiated for a user shader

#ifdef __CUDACC__
namespace sg {

// A user vertex shader on one vertex: its input registers to the position
// and the NA varyings.
template <class UVS, int NA>
__device__ void user_vs(DrawParams const& D, v4 const* in, v4* out) {
  salvia_gb300::vs_input vin;
  for (int r = 0; r < SG_MAX_VS_INPUTS; ++r) vin.attr[r] = salvia_gb300::detail::to_vec4(in[r]);
  salvia_gb300::vs_output vout;
  UVS vs;
  salvia_gb300::detail::shader_access::bind(vs, &D);
  vs.shader_prog(vin, vout);
  out[0] = mk4(vout.position.x, vout.position.y, vout.position.z, vout.position.w);
  for (int i = 0; i < NA; ++i) out[1 + i] = mk4(vout.attr[i].x, vout.attr[i].y, vout.attr[i].z, vout.attr[i].w);
}

// A user blend shader on one sample: ps_output from the fragment's colours.
template <class UBS>
__device__ void user_blend(TargetParams const& T, DrawParams const& D, uint32_t x, uint32_t y, uint32_t s, v4 src,
                           float4 const* more) {
  salvia_gb300::ps_output in;
  in.color[0] = salvia_gb300::vec4(src.x, src.y, src.z, src.w);
  for (uint32_t i = 0; i + 1 < SG_MAX_COLOR_TARGETS; ++i)
    if (more && i < T.nmore) in.color[i + 1] = salvia_gb300::vec4(more[i].x, more[i].y, more[i].z, more[i].w);
  UBS bs;
  salvia_gb300::detail::shader_access::bind(bs, &D);
  salvia_gb300::pixel_accessor acc;
  salvia_gb300::detail::shader_access::bind(acc, &T, x, y);
  bs.shader_prog(s, acc, in);
}

// Pixel shading of the fragments of shade key `key` with the user pixel
// shader UPS: interpolation as k_shade does it, the body per pixel, the
// quad's pass mask as cpp_pixel_shader::execute builds it.
template <class UPS>
__global__ void __launch_bounds__(256) k_shade_user(PassParams P, uint32_t key) {
  if ((P.counters->overflow & OVF_FATAL) || pass_gated(P)) return;
  uint32_t const nfrag = min(P.counters->chunk_total, P.chunk_capacity) * FRAG_CHUNK;
  int const q = threadIdx.x & 3;
  uint32_t const groups = gridDim.x * (blockDim.x >> 2);
  uint32_t const start = blockIdx.x * (blockDim.x >> 2) + (threadIdx.x >> 2);
  uint32_t base = 0, n = 0;
  if (P.frag_list) {
    for (uint32_t k = 0; k < key; ++k) base += P.class_counts[k];
    n = P.class_counts[key];
  }
  uint32_t const total = P.frag_list ? n : nfrag;
  uint32_t const rounds = (total + groups - 1) / groups;
  for (uint32_t it = 0; it < rounds; ++it) {
    uint32_t const idx = start + it * groups;
    uint32_t f;
    bool live;
    if (P.frag_list) {
      live = idx < total;
      f = live ? P.frag_list[base + idx] : 0u;
    } else {
      f = idx;
      live = f < nfrag && (f % FRAG_CHUNK) < P.chunk_count[f / FRAG_CHUNK];
    }
    uint32_t const pos = live ? P.frag_pos[f] : 0u;
    live = live && (pos >> 25) == key;
    uint32_t draw = 0xFFFFFFFFu;
    if (live) {
      uint32_t const rec = P.frag_rec[f], masks = P.frag_mask[f];
      DrawParams const& D = P.draws[rec_draw(P.recs + rec)];
      draw = rec_draw(P.recs + rec);
      TargetParams const& T = P.targets[D.target];
      salvia_gb300::detail::ps_device_ctx c;
      c.t = TriView{P.recs + rec, 1 + static_cast<int>(D.nattr)};
      c.D = &D;
      c.front = c.t.front();
      c.pixel = q;
      uint32_t const qx = (pos & 0xFFFu) << 1, qy = ((pos >> 12) & 0xFFFu) << 1;
      bool const full = (pos >> 24) & 1u;
      v4 const v0p = c.t.v0(0);
      c.dx = 0.5f + static_cast<float>(qx) - v0p.x;
      c.dy = 0.5f + static_cast<float>(qy) - v0p.y;
      c.centroid = !full && D.has_centroid;
      uint64_t const cov = expand_mask(masks >> 16);  // coverage before early-Z (rasterizer.cpp:1373)
      for (int p = 0; p < 4; ++p) {
        c.invw[p] = 1.0f / quad_pos(c.t, c.dx, c.dy, p).w;
        c.pdx[p] = c.dx + static_cast<float>(p & 1);
        c.pdy[p] = c.dy + static_cast<float>(p >> 1);
        uint32_t const pm = static_cast<uint32_t>(cov >> (16 * p)) & 0xFFFFu, fm = (1u << T.samples) - 1u;
        if (c.centroid && pm != fm && pm != 0) {
          float cx = 0.0f, cy = 0.0f;
          int cnt = 0;
          for (uint32_t s = 0; s < T.samples; ++s)
            if (pm & (1u << s)) {
              cx += T.sp_x[s];
              cy += T.sp_y[s];
              ++cnt;
            }
          float const inv = 1.0f / static_cast<float>(cnt);
          cx *= inv;
          cy *= inv;
          c.pdx[p] += cx - 0.5f;
          c.pdy[p] += cy - 0.5f;
        }
      }
      salvia_gb300::vs_output in;
      in.position = salvia_gb300::detail::to_vec4(quad_pos(c.t, c.dx, c.dy, q));
      for (int i = 0; i < SG_MAX_VARYINGS; ++i)
        in.attr[i] = salvia_gb300::detail::to_vec4(salvia_gb300::detail::pixel_attr(c, i, q));
      salvia_gb300::ps_output out;
      UPS ps;
      salvia_gb300::detail::shader_access::bind(ps, &c);
      bool const keep = ps.shader_prog(in, out);
      salvia_gb300::vec4 const o = out.color[0];
      P.frag_color[static_cast<size_t>(f) * 4 + q] = make_float4(o.x, o.y, o.z, o.w);
      if (P.frag_color_more)  // (a fixed trip count: out stays in registers)
#pragma unroll
        for (uint32_t i = 0; i + 1 < SG_MAX_COLOR_TARGETS; ++i)
          if (i < P.more_colors) {
            salvia_gb300::vec4 const m = out.color[i + 1];
            P.frag_color_more[(static_cast<size_t>(f) * 4 + q) * P.more_colors + i] = make_float4(m.x, m.y, m.z, m.w);
          }
      // the pass mask from int shifts of 0xFFFF by 16 i (cpp_pixel_shader.cpp:
      // 62-74): pixel 0 kept when pixel 0 or 2 passes, pixels 1-3 when 1 or 3 do
      int const qb = (threadIdx.x & 31) & ~3;
      uint32_t const passed = (__ballot_sync(0xFu << qb, keep) >> qb) & 0xFu;
      uint32_t const kept = ((passed & 5u) ? 1u : 0u) | ((passed & 10u) ? 14u : 0u);
      if (q == 0) P.frag_ps[f] = static_cast<uint8_t>(kept);
    }
    // ps_invocations: 4 per quad, counted per draw (one lane per quad)
    uint32_t const k = q == 0 ? draw : 0xFFFFFFFFu;
    uint32_t const grp = __match_any_sync(0xFFFFFFFFu, k);
    if (k != 0xFFFFFFFFu && (threadIdx.x & 31) == static_cast<uint32_t>(__ffs(grp) - 1))
      atomicAdd(&P.draw_stats[k].ps_invocations, 4ull * static_cast<unsigned>(__popc(grp)));
  }
}

// The output merger with the user blend shader UBS for the pass's user-blend draws.
template <class UBS>
__global__ void __launch_bounds__(RASTER_THREADS) k_merge_user(PassParams P) {
  merge_pass<UBS>(P);
}

}  // namespace sg

// Per-module device state: each module carries its own copy of the
// sampler's EWA weight table (a __constant__ of sg_common.cuh).
#define SALVIA_GB300_MODULE_INIT_(cls)                                                                          \
  static int32_t salvia_gb300_init_##cls(const float* ewa, void* stream) {                                    \
    return cudaMemcpyToSymbolAsync(sg::c_ewa, ewa, 256 * sizeof(float), 0, cudaMemcpyHostToDevice,            \
                                   static_cast<cudaStream_t>(stream)) == cudaSuccess                           \
               ? 0                                                                                             \
               : 1;                                                                                            \
  }

// Exports a vertex-shader class as extern "C" salvia_gb300_module_<cls>():
// the pass's geometry kernel instantiated for it (every draw of the pass; a
// pass holds one user vertex shader).
#define SALVIA_GB300_VERTEX_SHADER(cls)                                                                        \
  SALVIA_GB300_MODULE_INIT_(cls)                                                                               \
  __global__ void __launch_bounds__(128) salvia_gb300_geometry_##cls(sg::PassParams P) {                     \
    sg::geometry_pass<cls>(P);                                                                                 \
  }                                                                                                            \
  static void salvia_gb300_launch_##cls(const void* pass, uint32_t, uint32_t grid, void* stream) {            \
    salvia_gb300_geometry_##cls<<<grid, 128, 0, static_cast<cudaStream_t>(stream)>>>(                         \
        *static_cast<sg::PassParams const*>(pass));                                                            \
  }                                                                                                            \
  SALVIA_GB300_HOST_VE_(cls)                                                                                  \
  extern "C" sg_shader_module const* salvia_gb300_module_##cls() {                                            \
    static sg_shader_module const m = {SG_SHADER_ABI_VERSION, SG_STAGE_VERTEX, #cls, salvia_gb300_init_##cls, \
                                       salvia_gb300_launch_##cls, nullptr, nullptr, salvia_gb300_host_##cls}; \
    return &m;                                                                                                 \
  }

// Exports a pixel-shader class as extern "C" salvia_gb300_module_<cls>().
#define SALVIA_GB300_PIXEL_SHADER(cls)                                                                         \
  SALVIA_GB300_MODULE_INIT_(cls)                                                                               \
  static void salvia_gb300_launch_##cls(const void* pass, uint32_t key, uint32_t grid, void* stream) {        \
    sg::k_shade_user<cls><<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(                              \
        *static_cast<sg::PassParams const*>(pass), key);                                                       \
  }                                                                                                            \
  SALVIA_GB300_HOST_PI_(cls)                                                                                  \
  extern "C" sg_shader_module const* salvia_gb300_module_##cls() {                                            \
    static sg_shader_module const m = {SG_SHADER_ABI_VERSION, SG_STAGE_PIXEL, #cls, salvia_gb300_init_##cls,  \
                                       salvia_gb300_launch_##cls, salvia_gb300_host_##cls, nullptr, nullptr};  \
    return &m;                                                                                                 \
  }

// Exports a blend-shader class as extern "C" salvia_gb300_module_<cls>().
#define SALVIA_GB300_BLEND_SHADER(cls)                                                                         \
  SALVIA_GB300_MODULE_INIT_(cls)                                                                               \
  static void salvia_gb300_launch_##cls(const void* pass, uint32_t, uint32_t grid, void* stream) {            \
    sg::k_merge_user<cls><<<grid, sg::RASTER_THREADS, 0, static_cast<cudaStream_t>(stream)>>>(                \
        *static_cast<sg::PassParams const*>(pass));                                                            \
  }                                                                                                            \
  SALVIA_GB300_HOST_BL_(cls)                                                                                  \
  extern "C" sg_shader_module const* salvia_gb300_module_##cls() {                                            \
    static sg_shader_module const m = {SG_SHADER_ABI_VERSION, SG_STAGE_BLEND, #cls, salvia_gb300_init_##cls,  \
                                       salvia_gb300_launch_##cls, nullptr, salvia_gb300_host_##cls, nullptr};  \
    return &m;                                                                                                 \
  }
#endif  // __CUDACC__

#ifndef __CUDACC__
// Host-only modules (no device entries), which CPU backends of the ABI
// register and run: the same bodies built by a host C++ compiler.
#define SALVIA_GB300_HOST_MODULE_(cls, stage, ps, bs, vs)                                                      \
  extern "C" sg_shader_module const* salvia_gb300_module_##cls() {                                            \
    static sg_shader_module const m = {SG_SHADER_ABI_VERSION, stage, #cls, nullptr, nullptr, ps, bs, vs};      \
    return &m;                                                                                                 \
  }
#define SALVIA_GB300_VERTEX_SHADER(cls) \
  SALVIA_GB300_HOST_VE_(cls)            \
  SALVIA_GB300_HOST_MODULE_(cls, SG_STAGE_VERTEX, nullptr, nullptr, salvia_gb300_host_##cls)
#define SALVIA_GB300_PIXEL_SHADER(cls) \
  SALVIA_GB300_HOST_PI_(cls)           \
  SALVIA_GB300_HOST_MODULE_(cls, SG_STAGE_PIXEL, salvia_gb300_host_##cls, nullptr, nullptr)
#define SALVIA_GB300_BLEND_SHADER(cls) \
  SALVIA_GB300_HOST_BL_(cls)           \
  SALVIA_GB300_HOST_MODULE_(cls, SG_STAGE_BLEND, nullptr, salvia_gb300_host_##cls, nullptr)
#endif
