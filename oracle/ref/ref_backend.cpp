// Reference-backed implementation of the salvia_gb300.h C ABI.
//
// ORACLE INFRASTRUCTURE -- used only to generate the golden fixtures under
// tests/golden/ and to pin the CPU restatement in oracle/sg_oracle.cpp.  It is
// compiled together with the reference renderer's own, unmodified sources
// (salvia/src/core, salvia/src/resource, eflib/src/math.cpp) by
// oracle/ref/Makefile into oracle/_ref/libsalvia_ref.so, and drives them
// through the reference's public API: create_benchmark_renderer()
// (salvia/src/core/renderer.cpp:37-39), create_buffer/create_tex2d/
// create_sampler, set_* state calls and draw/draw_index
// (salvia/include/salvia/core/renderer.h:42-147).
//
// The stock shader programs of the ABI are written here as the reference's
// own cpp_vertex_shader / cpp_pixel_shader / cpp_blend_shader subclasses
// (salvia/include/salvia/core/shader.h:159-215), using the reference's math
// (eflib::transform, cpp_pixel_shader::tex2d, sampler::sample_2d_grad,
// salvia::lerp).
#include "salvia_gb300.h"

#include <salvia/core/async_object.h>
#include <salvia/core/framebuffer.h>
#include <salvia/core/raster_state.h>
#include <salvia/core/renderer.h>
#include <salvia/core/shader.h>
#include <salvia/resource/buffer.h>
#include <salvia/resource/input_layout.h>
#include <salvia/resource/pixel_accessor.h>
#include <salvia/resource/sampler.h>
#include <salvia/resource/surface.h>
#include <salvia/resource/texture.h>
#include <salvia/shader/shader_regs.h>

#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

using namespace salvia;
using namespace salvia::core;
using namespace salvia::resource;
using namespace salvia::shader;
using eflib::mat44;
using eflib::vec2;
using eflib::vec4;

namespace {

mat44 load_mat(float const* k) {
  return mat44(k[0], k[1], k[2], k[3], k[4], k[5], k[6], k[7], k[8], k[9], k[10], k[11], k[12],
               k[13], k[14], k[15]);
}

char const* semantic_name(uint32_t s) {
  switch (s) {
  case SG_SEMANTIC_POSITION: return "POSITION";
  case SG_SEMANTIC_COLOR: return "COLOR";
  case SG_SEMANTIC_NORMAL: return "NORMAL";
  default: return "TEXCOORD";
  }
}

class ref_vs : public cpp_vertex_shader {
public:
  sg_shader prog{};
  uint32_t nvary = 0;
  uint32_t mods[SG_MAX_VARYINGS] = {};
  sampler_ptr samp;

  ref_vs(sg_draw_desc const& d, sampler_ptr const& s) : prog(d.vs), nvary(d.num_varyings), samp(s) {
    for (uint32_t i = 0; i < SG_MAX_VARYINGS; ++i) mods[i] = d.varying_modifiers[i];
    for (uint32_t r = 0; r < d.num_inputs; ++r) {
      bind_semantic(semantic_name(d.inputs[r].semantic), d.inputs[r].semantic_index, r);
    }
  }

  sg_shader_module const* user = nullptr;  // a user vertex shader's module

  // the reference's sampler::sample for a user body's vertex texture fetch
  static void io_sample(void* b, float u, float v, float lod, float out[4]) {
    color_rgba32f const c = static_cast<ref_vs*>(b)->samp->sample(u, v, lod);
    out[0] = c.r;
    out[1] = c.g;
    out[2] = c.b;
    out[3] = c.a;
  }

  void shader_prog(vs_input const& in, vs_output& out) override {
    if (user) {  // the user body, compiled for the host
      sg_host_vs_io io{};
      for (uint32_t r = 0; r < SG_MAX_VS_INPUTS; ++r)
        for (int k = 0; k < 4; ++k) io.in[r][k] = in.attribute(r)[k];
      io.num_varyings = nvary;
      io.constants = prog.constants;
      io.backend = this;
      io.sample = io_sample;
      user->host_vs(&io);
      out.position() = vec4(io.position[0], io.position[1], io.position[2], io.position[3]);
      for (uint32_t i = 0; i < nvary; ++i) out.attribute(i) = vec4(io.attr[i][0], io.attr[i][1], io.attr[i][2], io.attr[i][3]);
      return;
    }
    mat44 m = load_mat(prog.constants);
    switch (prog.program) {
    case SG_VS_TRANSFORM:
      eflib::transform(out.position(), in.attribute(0), m);
      for (uint32_t i = 0; i < nvary; ++i) out.attribute(i) = in.attribute(i + 1);
      break;
    case SG_VS_MORPH_DISPLACE: {
      float w = prog.constants[16];
      float scale = prog.constants[17];
      vec4 p = in.attribute(0) + (in.attribute(1) - in.attribute(0)) * w;
      vec4 n = in.attribute(2);
      float h = samp->sample(in.attribute(3).x(), in.attribute(3).y(), 0.0f).r;
      float hs = h * scale;
      p[0] = p[0] + n[0] * hs;
      p[1] = p[1] + n[1] * hs;
      p[2] = p[2] + n[2] * hs;
      eflib::transform(out.position(), p, m);
      if (nvary > 0) out.attribute(0) = in.attribute(3);
      if (nvary > 1) out.attribute(1) = n;
      break;
    }
    default: break;
    }
  }
  uint32_t num_output_attributes() const override { return nvary; }
  uint32_t output_attribute_modifiers(uint32_t i) const override {
    return i < SG_MAX_VARYINGS ? mods[i] : vs_output::am_linear;
  }
  cpp_shader_ptr clone() override { return cpp_shader_ptr(new ref_vs(*this)); }
};

class ref_ps : public cpp_pixel_shader {
public:
  sg_shader prog{};
  sampler_ptr samp;

  ref_ps(sg_shader const& p, sampler_ptr const& s) : prog(p), samp(s) {}

  uint32_t nattr = 0;
  sg_shader_module const* user = nullptr;  // a user pixel shader's module

  // the reference's own cpp_pixel_shader helpers, for a user body's host io
  static void put(vec4 const& v, float out[4]) {
    for (int k = 0; k < 4; ++k) out[k] = v[k];
  }
  static void io_ddx(void* b, uint32_t reg, float out[4]) { put(static_cast<ref_ps*>(b)->ddx(reg), out); }
  static void io_ddy(void* b, uint32_t reg, float out[4]) { put(static_cast<ref_ps*>(b)->ddy(reg), out); }
  static void io_tex2d(void* b, uint32_t reg, float out[4]) {
    auto* p = static_cast<ref_ps*>(b);
    put(p->tex2d(*p->samp, reg).get_vec4(), out);
  }
  static void io_tex2dlod(void* b, uint32_t reg, float out[4]) {
    auto* p = static_cast<ref_ps*>(b);
    put(p->tex2dlod(*p->samp, reg).get_vec4(), out);
  }
  static void io_tex2dproj(void* b, uint32_t reg, float out[4]) {
    auto* p = static_cast<ref_ps*>(b);
    put(p->tex2dproj(*p->samp, reg).get_vec4(), out);
  }
  static void io_sample(void* b, float u, float v, float lod, float out[4]) {
    put(static_cast<ref_ps*>(b)->samp->sample(u, v, lod).get_vec4(), out);
  }
  static void io_sample_grad(void* b, float u, float v, float dxu, float dxv, float dyu, float dyv, float out[4]) {
    put(static_cast<ref_ps*>(b)->samp->sample_2d_grad(vec2(u, v), vec2(dxu, dxv), vec2(dyu, dyv), 0.0f).get_vec4(),
        out);
  }
  static void io_sample_cube(void* b, float x, float y, float z, float lod, float out[4]) {
    put(static_cast<ref_ps*>(b)->samp->sample_cube(x, y, z, lod).get_vec4(), out);
  }
  bool run_user(vs_output const& in, ps_output& out) {
    sg_host_ps_io io{};
    for (uint32_t a = 0; a < SG_MAX_VARYINGS && a < nattr; ++a)
      for (int k = 0; k < 4; ++k) io.attr[a][k] = in.attribute(a)[k];
    for (int k = 0; k < 4; ++k) io.position[k] = in.position()[k];
    io.front_face = front_face() ? 1u : 0u;
    io.num_varyings = nattr;
    io.constants = prog.constants;
    io.backend = this;
    io.ddx = io_ddx;
    io.ddy = io_ddy;
    io.tex2d = io_tex2d;
    io.tex2dlod = io_tex2dlod;
    io.tex2dproj = io_tex2dproj;
    io.sample = io_sample;
    io.sample_grad = io_sample_grad;
    io.sample_cube = io_sample_cube;
    bool const keep = user->host_ps(&io) != 0;
    for (uint32_t i = 0; i < SG_MAX_COLOR_TARGETS; ++i)
      out.color[i] = vec4(io.color[i][0], io.color[i][1], io.color[i][2], io.color[i][3]);
    return keep;
  }

  bool shader_prog(vs_output const& in, ps_output& out) override {
    if (user) return run_user(in, out);
    switch (prog.program) {
    case SG_PS_COLOR: out.color[0] = in.attribute(0); return true;
    case SG_PS_COLOR_MRT:
      for (uint32_t i = 0; i < SG_MAX_COLOR_TARGETS; ++i) out.color[i] = i < nattr ? in.attribute(i) : vec4(0, 0, 0, 0);
      return true;
    case SG_PS_CONSTANT:
      out.color[0] = vec4(prog.constants[0], prog.constants[1], prog.constants[2], prog.constants[3]);
      return true;
    case SG_PS_TEX_MODULATE: {
      color_rgba32f c = tex2d(*samp, 0);
      out.color[0] = c.get_vec4() * in.attribute(1);
      return true;
    }
    case SG_PS_TEX_GRAD_MODULATE: {
      vec4 dx = ddx(0);
      vec4 dy = ddy(0);
      vec2 uv(in.attribute(0).x(), in.attribute(0).y());
      color_rgba32f c =
          samp->sample_2d_grad(uv, vec2(dx.x(), dx.y()), vec2(dy.x(), dy.y()), 0.0f);
      out.color[0] = c.get_vec4() * in.attribute(1);
      return true;
    }
    case SG_PS_TEX_LOD_MODULATE: out.color[0] = tex2dlod(*samp, 0).get_vec4() * in.attribute(1); return true;
    case SG_PS_TEXCUBE_MODULATE: {
      vec4 const& a = in.attribute(0);
      out.color[0] = samp->sample_cube(a[0], a[1], a[2], a[3]).get_vec4() * in.attribute(1);
      return true;
    }
    case SG_PS_TEX_PROJ_MODULATE: out.color[0] = tex2dproj(*samp, 0).get_vec4() * in.attribute(1); return true;
    case SG_PS_TEX_ALPHA_TEST: {
      vec4 c = tex2d(*samp, 0).get_vec4() * in.attribute(1);
      out.color[0] = c;
      return !(c[3] < prog.constants[0]);
    }
    default: out.color[0] = vec4(0, 0, 0, 0); return true;
    }
  }
  cpp_shader_ptr clone() override { return cpp_shader_ptr(new ref_ps(*this)); }
};

class ref_bs : public cpp_blend_shader {
public:
  uint32_t program;
  uint32_t ncolor = 1;
  sg_shader_module const* user = nullptr;  // a user blend shader's module
  float constants[SG_MAX_SHADER_CONSTANTS] = {};
  explicit ref_bs(uint32_t p) : program(p) {}
  static void io_get(void* b, uint32_t t, uint32_t s, float out[4]) {
    color_rgba32f c = static_cast<pixel_accessor*>(b)->color(t, s);
    vec4 v = c.get_vec4();
    for (int k = 0; k < 4; ++k) out[k] = v[k];
  }
  static void io_set(void* b, uint32_t t, uint32_t s, const float c[4]) {
    static_cast<pixel_accessor*>(b)->color(t, s, color_rgba32f(c[0], c[1], c[2], c[3]));
  }
  bool shader_prog(size_t sample, pixel_accessor& inout, ps_output const& in) override {
    if (user) {  // the user body on the reference's pixel_accessor
      sg_host_bs_io io{};
      io.sample = static_cast<uint32_t>(sample);
      for (uint32_t i = 0; i < SG_MAX_COLOR_TARGETS; ++i)
        for (int k = 0; k < 4; ++k) io.in_color[i][k] = in.color[i][k];
      io.constants = constants;
      io.backend = &inout;
      io.get = io_get;
      io.set = io_set;
      return user->host_bs(&io) != 0;
    }
    switch (program) {
    case SG_BS_REPLACE_ALL:
      for (uint32_t i = 0; i < ncolor; ++i) inout.color(i, sample, color_rgba32f(in.color[i]));
      break;
    case SG_BS_LERP_SRC_ALPHA: {
      color_rgba32f dst = inout.color(0, sample);
      color_rgba32f src(in.color[0]);
      inout.color(0, sample, lerp(dst, src, in.color[0][3]));
      break;
    }
    case SG_BS_ADD: {
      color_rgba32f dst = inout.color(0, sample);
      inout.color(0, sample, color_rgba32f(dst.get_vec4() + in.color[0]));
      break;
    }
    default: inout.color(0, sample, color_rgba32f(in.color[0])); break;
    }
    return true;
  }
  cpp_shader_ptr clone() override { return cpp_shader_ptr(new ref_bs(*this)); }
};

}  // namespace

struct sg_device {
  renderer_ptr r;
  uint32_t next = 1;
  std::map<uint32_t, buffer_ptr> buffers;
  std::map<uint32_t, texture_ptr> textures;
  std::map<uint32_t, sampler_ptr> samplers;
  std::vector<sg_shader_module const*> user_shaders;  // program SG_USER_PROGRAM_BASE + i
};

extern "C" {

int32_t sg_shader_register(sg_device* d, const sg_shader_module* m, uint32_t* out) {
  if (!d || !m || !out || m->abi_version != SG_SHADER_ABI_VERSION ||
      (m->stage == SG_STAGE_PIXEL && !m->host_ps) || (m->stage == SG_STAGE_BLEND && !m->host_bs) ||
      (m->stage == SG_STAGE_VERTEX && !m->host_vs) ||
      (m->stage != SG_STAGE_PIXEL && m->stage != SG_STAGE_BLEND && m->stage != SG_STAGE_VERTEX))
    return SG_INVALID_PARAMETER;
  for (size_t i = 0; i < d->user_shaders.size(); ++i)
    if (d->user_shaders[i] == m) {
      *out = SG_USER_PROGRAM_BASE + static_cast<uint32_t>(i);
      return SG_OK;
    }
  d->user_shaders.push_back(m);
  *out = SG_USER_PROGRAM_BASE + static_cast<uint32_t>(d->user_shaders.size() - 1);
  return SG_OK;
}

int32_t sg_device_create(int32_t, void*, sg_device** out) {
  auto* d = new sg_device();
  d->r = create_benchmark_renderer();
  *out = d;
  return SG_OK;
}
void sg_device_destroy(sg_device* d) { delete d; }
int32_t sg_sync(sg_device* d) {
  d->r->flush();
  return SG_OK;
}
const char* sg_last_error(sg_device*) { return ""; }

int32_t sg_buffer_create(sg_device* d, size_t size, uint32_t* out) {
  auto b = d->r->create_buffer(size);
  *out = d->next++;
  d->buffers[*out] = b;
  return SG_OK;
}
int32_t sg_buffer_upload(sg_device* d, uint32_t b, size_t off, const void* src, size_t size) {
  auto it = d->buffers.find(b);
  if (it == d->buffers.end() || off + size > it->second->size()) return SG_INVALID_PARAMETER;
  std::memcpy(it->second->raw_data(off), src, size);
  return SG_OK;
}
int32_t sg_buffer_download(sg_device* d, uint32_t b, size_t off, void* dst, size_t size) {
  auto it = d->buffers.find(b);
  if (it == d->buffers.end() || off + size > it->second->size()) return SG_INVALID_PARAMETER;
  std::memcpy(dst, it->second->raw_data(off), size);
  return SG_OK;
}
int32_t sg_buffer_destroy(sg_device* d, uint32_t b) {
  d->buffers.erase(b);
  return SG_OK;
}

int32_t sg_texture_create(sg_device* d, uint32_t w, uint32_t h, uint32_t s, uint32_t fmt,
                          uint32_t* out) {
  if (fmt > SG_FMT_R32I) return SG_INVALID_PARAMETER;
  auto t = d->r->create_tex2d(w, h, s, static_cast<pixel_format>(fmt));
  *out = d->next++;
  d->textures[*out] = t;
  return SG_OK;
}
int32_t sg_texture_create_cube(sg_device* d, uint32_t w, uint32_t h, uint32_t s, uint32_t fmt, uint32_t* out) {
  if (fmt > SG_FMT_R32I) return SG_INVALID_PARAMETER;
  auto t = d->r->create_texcube(w, h, s, static_cast<pixel_format>(fmt));
  *out = d->next++;
  d->textures[*out] = t;
  return SG_OK;
}
static surface* tex_level(sg_device* d, uint32_t t, uint32_t level) {
  auto it = d->textures.find(t);
  if (it == d->textures.end()) return nullptr;
  return it->second->subresource(level).get();
}
int32_t sg_texture_upload(sg_device* d, uint32_t t, uint32_t level, const void* src, size_t size) {
  surface* s = tex_level(d, t, level);
  // a cube's faces 1-5 are unreachable in the reference (texture_cube leaves
  // its LOD range at [0, 0], so subresources past 0 are null): dropped
  auto it = d->textures.find(t);
  if (!s && it != d->textures.end() && it->second->get_texture_type() == texture_type_cube && level < 6) return SG_OK;
  if (!s || size != s->pitch() * s->height()) return SG_INVALID_PARAMETER;
  std::memcpy(s->texel_address(0, 0, 0), src, size);
  return SG_OK;
}
int32_t sg_texture_download(sg_device* d, uint32_t t, uint32_t level, void* dst, size_t size) {
  surface* s = tex_level(d, t, level);
  if (!s || size != s->pitch() * s->height()) return SG_INVALID_PARAMETER;
  std::memcpy(dst, s->texel_address(0, 0, 0), size);
  return SG_OK;
}
int32_t sg_texture_gen_mipmap(sg_device* d, uint32_t t, uint32_t filter) {
  auto it = d->textures.find(t);
  if (it == d->textures.end()) return SG_INVALID_PARAMETER;
  it->second->gen_mipmap(static_cast<filter_type>(filter), true);
  return SG_OK;
}
int32_t sg_texture_info(sg_device* d, uint32_t t, uint32_t level, uint32_t* w, uint32_t* h,
                        uint32_t* s, uint32_t* fmt, uint32_t* levels) {
  auto it = d->textures.find(t);
  if (it == d->textures.end()) return SG_INVALID_PARAMETER;
  surface* sf = it->second->subresource(level).get();
  if (!sf) return SG_INVALID_PARAMETER;
  if (w) *w = static_cast<uint32_t>(sf->width());
  if (h) *h = static_cast<uint32_t>(sf->height());
  if (s) *s = static_cast<uint32_t>(sf->sample_count());
  if (fmt) *fmt = static_cast<uint32_t>(sf->get_pixel_format());
  if (levels) *levels = static_cast<uint32_t>(it->second->min_lod() + 1);
  return SG_OK;
}
int32_t sg_texture_destroy(sg_device* d, uint32_t t) {
  d->textures.erase(t);
  return SG_OK;
}

int32_t sg_sampler_create(sg_device* d, const sg_sampler_desc* sd, uint32_t tex, uint32_t* out) {
  auto it = d->textures.find(tex);
  if (it == d->textures.end()) return SG_INVALID_PARAMETER;
  sampler_desc desc;
  desc.min_filter = static_cast<filter_type>(sd->min_filter);
  desc.mag_filter = static_cast<filter_type>(sd->mag_filter);
  desc.mip_filter = static_cast<filter_type>(sd->mip_filter);
  desc.mip_qual = static_cast<mip_quality>(sd->mip_quality);
  desc.addr_mode_u = static_cast<address_mode>(sd->address_u);
  desc.addr_mode_v = static_cast<address_mode>(sd->address_v);
  desc.addr_mode_w = static_cast<address_mode>(sd->address_w);
  desc.mip_lod_bias = sd->lod_bias;
  desc.max_anisotropy = sd->max_anisotropy;
  desc.border_color = color_rgba32f(sd->border_color[0], sd->border_color[1], sd->border_color[2],
                                    sd->border_color[3]);
  desc.min_lod = sd->min_lod;
  desc.max_lod = sd->max_lod;
  *out = d->next++;
  d->samplers[*out] = d->r->create_sampler(desc, it->second);
  return SG_OK;
}
int32_t sg_sampler_destroy(sg_device* d, uint32_t s) {
  d->samplers.erase(s);
  return SG_OK;
}

int32_t sg_draw(sg_device* d, const sg_draw_desc* desc, sg_draw_stats* stats) {
  auto& r = d->r;
  sampler_ptr vs_samp = desc->vs.samplers[0] ? d->samplers[desc->vs.samplers[0]] : sampler_ptr();
  sampler_ptr ps_samp = desc->ps.samplers[0] ? d->samplers[desc->ps.samplers[0]] : sampler_ptr();
  auto vs = std::make_shared<ref_vs>(*desc, vs_samp);
  auto ps = std::make_shared<ref_ps>(desc->ps, ps_samp);
  auto bs = std::make_shared<ref_bs>(desc->bs.program);

  std::vector<input_element_desc> elems;
  for (uint32_t i = 0; i < desc->num_inputs; ++i) {
    auto const& in = desc->inputs[i];
    elems.emplace_back(semantic_name(in.semantic), in.semantic_index,
                       static_cast<format>(in.format), in.slot, in.offset, input_per_vertex, 0);
  }
  auto layout = r->create_input_layout(elems.data(), elems.size(), cpp_vertex_shader_ptr(vs));

  std::vector<buffer_ptr> bufs(desc->num_streams);
  std::vector<size_t> strides(desc->num_streams), offsets(desc->num_streams);
  for (uint32_t i = 0; i < desc->num_streams; ++i) {
    bufs[i] = d->buffers[desc->streams[i].buffer];
    strides[i] = desc->streams[i].stride;
    offsets[i] = desc->streams[i].offset;
  }
  if (desc->num_streams)
    r->set_vertex_buffers(0, desc->num_streams, bufs.data(), strides.data(), offsets.data());
  if (desc->indexed)
    r->set_index_buffer(d->buffers[desc->index_buffer], static_cast<format>(desc->index_format));
  r->set_input_layout(layout);
  r->set_primitive_topology(static_cast<primitive_topology>(desc->topology));
  r->set_vertex_shader(vs);
  r->set_pixel_shader(ps);
  r->set_blend_shader(bs);

  raster_desc rd;
  rd.fm = static_cast<fill_mode>(desc->raster.fill_mode);
  rd.cm = static_cast<cull_mode>(desc->raster.cull_mode);
  rd.front_ccw = desc->raster.front_ccw != 0;
  r->set_rasterizer_state(std::make_shared<raster_state>(rd));

  depth_stencil_desc dsd;
  auto const& s = desc->depth_stencil;
  dsd.depth_enable = s.depth_enable != 0;
  dsd.depth_write_mask = s.depth_write != 0;
  dsd.depth_func = static_cast<compare_function>(s.depth_func);
  dsd.stencil_enable = s.stencil_enable != 0;
  dsd.stencil_read_mask = static_cast<uint8_t>(s.stencil_read_mask);
  dsd.stencil_write_mask = static_cast<uint8_t>(s.stencil_write_mask);
  dsd.front_face.stencil_fail_op = static_cast<stencil_op>(s.front.fail_op);
  dsd.front_face.stencil_depth_fail_op = static_cast<stencil_op>(s.front.depth_fail_op);
  dsd.front_face.stencil_pass_op = static_cast<stencil_op>(s.front.pass_op);
  dsd.front_face.stencil_func = static_cast<compare_function>(s.front.func);
  dsd.back_face.stencil_fail_op = static_cast<stencil_op>(s.back.fail_op);
  dsd.back_face.stencil_depth_fail_op = static_cast<stencil_op>(s.back.depth_fail_op);
  dsd.back_face.stencil_pass_op = static_cast<stencil_op>(s.back.pass_op);
  dsd.back_face.stencil_func = static_cast<compare_function>(s.back.func);
  r->set_depth_stencil_state(std::make_shared<depth_stencil_state>(dsd), desc->stencil_ref);

  std::vector<surface_ptr> colors;
  if (desc->color_target) {
    colors.push_back(d->textures[desc->color_target]->subresource(0));
    for (uint32_t i = 0; i + 1 < SG_MAX_COLOR_TARGETS && desc->more_color_targets[i]; ++i)
      colors.push_back(d->textures[desc->more_color_targets[i]]->subresource(0));
  }
  ps->nattr = desc->num_varyings;
  if (desc->vs.program >= SG_USER_PROGRAM_BASE) {
    if (desc->vs.program - SG_USER_PROGRAM_BASE >= d->user_shaders.size()) return SG_INVALID_PARAMETER;
    vs->user = d->user_shaders[desc->vs.program - SG_USER_PROGRAM_BASE];
  }
  if (desc->ps.program >= SG_USER_PROGRAM_BASE) {
    if (desc->ps.program - SG_USER_PROGRAM_BASE >= d->user_shaders.size()) return SG_INVALID_PARAMETER;
    ps->user = d->user_shaders[desc->ps.program - SG_USER_PROGRAM_BASE];
  }
  if (desc->bs.program >= SG_USER_PROGRAM_BASE) {
    if (desc->bs.program - SG_USER_PROGRAM_BASE >= d->user_shaders.size()) return SG_INVALID_PARAMETER;
    bs->user = d->user_shaders[desc->bs.program - SG_USER_PROGRAM_BASE];
    std::memcpy(bs->constants, desc->bs.constants, sizeof(bs->constants));
  }
  bs->ncolor = static_cast<uint32_t>(std::max<size_t>(1, colors.size()));
  surface_ptr ds = desc->ds_target ? d->textures[desc->ds_target]->subresource(0) : surface_ptr();
  if (r->set_render_targets(colors.size(), colors.empty() ? nullptr : colors.data(), ds) != result::ok)
    return SG_FAILED;
  viewport vp{desc->viewport.x, desc->viewport.y, desc->viewport.w,
              desc->viewport.h, desc->viewport.minz, desc->viewport.maxz};
  r->set_viewport(vp);

  async_object_ptr q_pipe, q_int;
  if (stats) {
    q_pipe = r->create_query(async_object_ids::pipeline_statistics);
    q_int = r->create_query(async_object_ids::internal_statistics);
    r->begin(q_pipe);
    r->begin(q_int);
  }
  result rv = desc->indexed ? r->draw_index(desc->start, desc->prim_count, desc->base_vertex)
                            : r->draw(desc->start, desc->prim_count);
  if (stats) {
    r->end(q_pipe);
    r->end(q_int);
    pipeline_statistics ps_stat{};
    internal_statistics in_stat{};
    r->get_data(q_pipe, &ps_stat, false);
    r->get_data(q_int, &in_stat, false);
    stats->ia_primitives = ps_stat.ia_primitives;
    stats->cprimitives = ps_stat.cprimitives;
    stats->ps_invocations = ps_stat.ps_invocations;
    stats->backend_input_pixels = in_stat.backend_input_pixels;
    stats->ia_vertices = ps_stat.ia_vertices;
    stats->vs_invocations = ps_stat.vs_invocations;
    stats->cinvocations = ps_stat.cinvocations;
  }
  r->flush();
  return rv == result::ok ? SG_OK : SG_FAILED;
}

int32_t sg_clear_color(sg_device* d, uint32_t t, const float rgba[4]) {
  auto it = d->textures.find(t);
  if (it == d->textures.end()) return SG_INVALID_PARAMETER;
  d->r->clear_color(it->second->subresource(0), color_rgba32f(rgba[0], rgba[1], rgba[2], rgba[3]));
  d->r->flush();
  return SG_OK;
}
int32_t sg_clear_depth_stencil(sg_device* d, uint32_t t, uint32_t flags, float depth,
                               uint32_t stencil) {
  auto it = d->textures.find(t);
  if (it == d->textures.end()) return SG_INVALID_PARAMETER;
  d->r->clear_depth_stencil(it->second->subresource(0), flags, depth, stencil);
  d->r->flush();
  return SG_OK;
}
int32_t sg_resolve(sg_device* d, uint32_t src, uint32_t dst) {
  auto a = d->textures.find(src), b = d->textures.find(dst);
  if (a == d->textures.end() || b == d->textures.end()) return SG_INVALID_PARAMETER;
  a->second->subresource(0)->resolve(*b->second->subresource(0));
  return SG_OK;
}

}  // extern "C"
