// User shader bodies for the tests: written as an application would write
// its own cpp_pixel_shader / cpp_blend_shader classes (shader.h:169-215),
// compiled with nvcc into a shader module (salvia_gb300/device_shader.cuh).
#include <salvia_gb300/device_shader.cuh>

using salvia_gb300::ps_output;
using salvia_gb300::vec4;
using salvia_gb300::vs_output;

// A tinted, alpha-tested texture lookup in the reference samples' style:
// tex2d of register 0 modulated by register 1, tinted by constants 0-2 with
// weight constant 3, a derivative-dependent term (the squared length of
// ddx and ddy of register 0, weight constant 4) added to blue, and the pixel
// discarded when the modulated alpha is below constant 5.
struct tinted_alpha_test_ps : salvia_gb300::pixel_shader {
  __host__ __device__ bool shader_prog(vs_output const& in, ps_output& out) const {
    vec4 const c = tex2d(0) * in.attribute(1);
    vec4 const tint(constant(0), constant(1), constant(2), 1.0f);
    vec4 o = salvia_gb300::lerp(c, c * tint, constant(3));
    vec4 const gx = ddx(0), gy = ddy(0);
    o.z = o.z + ((gx.x * gx.x + gx.y * gx.y) + (gy.x * gy.x + gy.y * gy.y)) * constant(4);
    out.color[0] = o;
    return !(c.w < constant(5));
  }
};
SALVIA_GB300_PIXEL_SHADER(tinted_alpha_test_ps)

// Projective lookup (tex2dproj) on the front faces, a level-of-detail lookup
// (tex2dlod of register 0) on the back faces.
struct proj_or_lod_ps : salvia_gb300::pixel_shader {
  __host__ __device__ bool shader_prog(vs_output const& in, ps_output& out) const {
    out.color[0] = (front_face() ? tex2dproj(0) : tex2dlod(0)) * in.attribute(1);
    return true;
  }
};
SALVIA_GB300_PIXEL_SHADER(proj_or_lod_ps)

// "Screen" blending with opacity constant 0: dst + src k - dst src k.
struct screen_blend_bs : salvia_gb300::blend_shader {
  __host__ __device__ bool shader_prog(size_t sample, salvia_gb300::pixel_accessor& inout, ps_output const& in) const {
    vec4 const dst = inout.color(0, static_cast<int>(sample));
    vec4 const src = in.color[0];
    float const k = constant(0);
    inout.color(0, static_cast<int>(sample), (dst + src * k) - (dst * src) * k);
    return true;
  }
};
SALVIA_GB300_BLEND_SHADER(screen_blend_bs)

// A vertex shader with a height-dependent shear and a vertex texture fetch:
// x += y^2 * constant(16), then the row-vector transform by the matrix in
// constants 0-15 (eflib::transform's dot products, left to right); the
// texture coordinate (register 1) passes through, and the colour (register
// 2) is modulated by the texel fetched at it (sampler::sample, level 0).
struct shear_fetch_vs : salvia_gb300::vertex_shader {
  __host__ __device__ void shader_prog(salvia_gb300::vs_input const& in, vs_output& out) const {
    vec4 p = in.attribute(0);
    p.x = p.x + (p.y * p.y) * constant(16);
    vec4 o;
    o.x = ((p.x * constant(0) + p.y * constant(4)) + p.z * constant(8)) + p.w * constant(12);
    o.y = ((p.x * constant(1) + p.y * constant(5)) + p.z * constant(9)) + p.w * constant(13);
    o.z = ((p.x * constant(2) + p.y * constant(6)) + p.z * constant(10)) + p.w * constant(14);
    o.w = ((p.x * constant(3) + p.y * constant(7)) + p.z * constant(11)) + p.w * constant(15);
    out.position = o;
    vec4 const uv = in.attribute(1);
    out.attribute(0) = uv;
    vec4 const t = sample(uv.x, uv.y, 0.0f);
    out.attribute(1) = in.attribute(2) * vec4(t.x, t.y, t.z, 1.0f);
  }
};
SALVIA_GB300_VERTEX_SHADER(shear_fetch_vs)
