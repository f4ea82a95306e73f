// renderer.hpp -- C++ renderer facade over the salvia_gb300.h C ABI.
//
// Apps written against Salvia's renderer interface
// (salvia/include/salvia/core/renderer.h:42-147) keep their structure when
// they include this header instead: the same class names in the same
// namespaces (salvia::core, salvia::resource), the same factories
// (create_benchmark_renderer / create_software_renderer), the same state
// objects (raster_state, depth_stencil_state, sampler, input_layout,
// viewport), the same draw / draw_index / clear / flush / query calls and
// the same `result` codes.  Everything forwards to the C ABI, so this header
// needs no CUDA headers and works with any library that exports the ABI
// (the GPU library, or the CPU oracle used by the tests).
//
// The one structural difference is the shaders.  The reference runs the
// virtual `shader_prog` of user C++ classes on the CPU (shader.h:159-215);
// device kernels cannot call host virtuals, so here a cpp_vertex_shader /
// cpp_pixel_shader / cpp_blend_shader names a compiled device program
// (`program()`) and carries its constants and samplers, declared exactly as
// the reference's cpp_shader_impl does (declare_constant, declare_sampler,
// bind_semantic, set_constant, set_sampler).  Stock classes cover the
// programs the library ships: the MVP vertex shader, colour / constant /
// texture pixel shaders and the replace / src-alpha / additive blends.
//
// Header-only, C++17.  Link with libsalvia_gb300.so.
#pragma once

#include <dlfcn.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <fstream>
#include <functional>
#include <map>
#include <memory>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../salvia_gb300.h"

namespace salvia {

// salvia/include/salvia/common/constants.h:9, plus the two codes the GPU adds
enum class result : uint32_t { ok, failed, out_of_memory, invalid_parameter, timeout, cuda_error };

enum map_mode {
  map_mode_none = 0, map_read = 1, map_write = 2, map_read_write = 3, map_write_discard = 4,
  map_write_no_overwrite = 5
};
enum primitive_topology {
  primitive_line_list = 0,
  primitive_line_strip = 1,
  primitive_triangle_list = 2,
  primitive_triangle_strip = 4
};
enum cull_mode { cull_none = 0, cull_front = 1, cull_back = 2 };
enum fill_mode { fill_wireframe = 0, fill_solid = 1 };
enum address_mode { address_wrap = 0, address_mirror = 1, address_clamp = 2, address_border = 3 };
enum filter_type { filter_point = 0, filter_linear = 1, filter_anisotropic = 2 };
enum mip_quality { mip_lo_quality = 0, mip_mi_quality = 1, mip_hi_quality = 2 };
enum compare_function {
  compare_function_never = 0, compare_function_less = 1, compare_function_equal = 2,
  compare_function_less_equal = 3, compare_function_greater = 4, compare_function_not_equal = 5,
  compare_function_greater_equal = 6, compare_function_always = 7
};
enum stencil_op {
  stencil_op_keep = 1, stencil_op_zero = 2, stencil_op_replace = 3, stencil_op_incr_sat = 4,
  stencil_op_decr_sat = 5, stencil_op_invert = 6, stencil_op_incr_wrap = 7, stencil_op_decr_wrap = 8
};
enum clear_flag { clear_depth = 0x1, clear_stencil = 0x2 };
enum class async_object_ids : uint32_t {
  none, event, occlusion, pipeline_statistics, occlusion_predicate, internal_statistics, pipeline_profiles, count
};
enum class async_status : uint32_t { error, timeout, ready };

// pixel formats (colors_convertors.h:39-45) and the GPU's three extensions
enum pixel_format {
  pixel_format_color_rgba32f = 0, pixel_format_color_rgb32f = 1, pixel_format_color_bgra8 = 2,
  pixel_format_color_rgba8 = 3, pixel_format_color_r32f = 4, pixel_format_color_rg32f = 5,
  pixel_format_color_r32i = 6,
  pixel_format_color_rgba16f = SG_FMT_RGBA16F, pixel_format_depth_d32f = SG_FMT_D32F,
  pixel_format_depth_d24s8 = SG_FMT_D24S8
};
// vertex / index formats (salvia/include/salvia/common/format.h)
enum format {
  format_unknown = 0, format_r32g32b32a32_float = 2, format_r32g32b32a32_sint = 4, format_r32g32b32_float = 6,
  format_r32g32_float = 16, format_r32_float = 41, format_r32_uint = 42, format_r16_uint = 57
};

inline result to_result(int32_t s) { return static_cast<result>(s); }

}  // namespace salvia

// Compiled SASL shaders (shader_object.h, renderer.h:136-147).  compile()
// translates the source with the GPU library's sg_sasl_translate into the
// class of a user shader module, builds that with nvcc (or, with
// SALVIA_GB300_SASL_HOST_ONLY set, the host body alone with the host
// compiler, for CPU backends of the ABI) into $SALVIA_GB300_SHADER_CACHE
// (default /tmp/salvia_gb300_shaders), loads it, and keeps the stage
// interface the translator reported.  The renderer binds such an object with
// set_vertex_shader_code / set_pixel_shader_code; its uniforms and samplers
// come from set_vs_variable / set_ps_variable / set_vs_sampler /
// set_ps_sampler by name.
namespace salvia::shader {
// constants.h:11-20
enum languages { lang_none, lang_general, lang_vertex_shader, lang_pixel_shader, lang_blending_shader, lang_count };
struct shader_profile {  // reflection.h:10-12
  languages language;
};

class shader_object {
public:
  struct io_item {
    std::string semantic;  // upper case, without the index
    uint32_t index;
    int32_t reg;  // register, link slot or colour target; -1 the position
    uint32_t comps;
  };
  struct uniform {
    std::string name;
    uint32_t word, words;
  };
  languages language = lang_none;
  std::string cls, source;
  std::vector<io_item> inputs, outputs;
  std::vector<uniform> uniforms;
  std::vector<std::string> samplers;
  uint32_t varyings = 0;
  sg_shader_module const* module = nullptr;
};
using shader_object_ptr = std::shared_ptr<shader_object>;
}  // namespace salvia::shader

namespace salvia::detail {
// the tree this header lies in: $SALVIA_GB300_ROOT, else three levels above it
inline std::string gb300_root() {
  if (char const* r = std::getenv("SALVIA_GB300_ROOT")) return r;
  std::string f = __FILE__;
  for (int i = 0; i < 3; ++i) {
    size_t const p = f.find_last_of('/');
    f = p == std::string::npos ? std::string(".") : f.substr(0, p);
  }
  return f;
}
// the translator: the linked library's, else the GPU library of the tree
inline void* sasl_library() {
  // (RTLD_DEFAULT is a null handle: the program's own handle searches the same scope)
  if (dlsym(RTLD_DEFAULT, "sg_sasl_translate")) return dlopen(nullptr, RTLD_NOW);
  static void* const h =
      dlopen((gb300_root() + "/salviarenderer_gb300/_lib/libsalvia_gb300.so").c_str(), RTLD_NOW | RTLD_LOCAL);
  return h;
}
inline std::string upper(std::string s) {
  for (char& c : s)
    if (c >= 'a' && c <= 'z') c = static_cast<char>(c - 'a' + 'A');
  return s;
}
inline bool same_semantic(std::string a, std::string b) {
  a = upper(a);
  b = upper(b);
  if (a == "SV_POSITION") a = "POSITION";
  if (b == "SV_POSITION") b = "POSITION";
  return a == b;
}
}  // namespace salvia::detail

namespace salvia::core {

struct vec4 {
  float x = 0, y = 0, z = 0, w = 0;
};
struct mat44 {  // row-major, m[r][c]; vertices are row vectors (clip = v x M)
  float m[4][4] = {};
  static mat44 identity() {
    mat44 r;
    for (int i = 0; i < 4; ++i) r.m[i][i] = 1.0f;
    return r;
  }
};
struct color_rgba32f {
  float r = 0, g = 0, b = 0, a = 0;
  color_rgba32f() = default;
  color_rgba32f(float r_, float g_, float b_, float a_) : r(r_), g(g_), b(b_), a(a_) {}
};

struct viewport {  // salvia/include/salvia/core/viewport.h
  float x, y, w, h, minz, maxz;
};

namespace detail {
// What a running query adds up (pipeline_statistics and internal_statistics,
// async_object.h:90-175).
struct query_counters {
  uint64_t ia_vertices = 0, ia_primitives = 0, vs_invocations = 0, cinvocations = 0, cprimitives = 0,
           ps_invocations = 0, backend_input_pixels = 0;
};

// Owns the C-ABI device; shared by the renderer and every resource it made,
// so a resource never outlives the device its handle belongs to.
//
// It also holds the renderer's queued commands.  The reference's renderer
// executes each call as it comes (the synchronous renderer) or queues it for
// a render thread (async_renderer.cpp:19-104); here draws, clears and
// resolves are queued and go to the device as one command list (sg_submit,
// which runs them exactly as one-by-one calls would, many draws per kernel
// chain) when something needs their results or changes what they read:
// flush() and get_data() on the renderer, any read, write, mip generation,
// resolve or destruction of a resource, or a full queue.  Errors of queued
// commands are therefore reported by the call that submits them.
struct device_ref {
  sg_device* dev = nullptr;
  explicit device_ref(sg_device* d) : dev(d) {}
  ~device_ref() {
    if (dev) {
      flush();
      sg_device_destroy(dev);
    }
  }
  device_ref(device_ref const&) = delete;
  device_ref& operator=(device_ref const&) = delete;

  static constexpr size_t max_queued = 1024;

  void queue_draw(sg_draw_desc const& d, std::vector<std::shared_ptr<query_counters>> const& queries) {
    descs_.push_back(d);
    sg_command c{};
    c.type = SG_CMD_DRAW;
    c.draw = &descs_.back();
    push(c, queries);
  }
  void queue_clear_color(uint32_t tex, float const rgba[4]) {
    sg_command c{};
    c.type = SG_CMD_CLEAR_COLOR;
    c.texture = tex;
    std::memcpy(c.color, rgba, sizeof(c.color));
    push(c, {});
  }
  void queue_clear_depth_stencil(uint32_t tex, uint32_t flags, float depth, uint32_t stencil) {
    sg_command c{};
    c.type = SG_CMD_CLEAR_DEPTH_STENCIL;
    c.texture = tex;
    c.flags = flags;
    c.depth = depth;
    c.stencil = stencil;
    push(c, {});
  }
  void queue_resolve(uint32_t src, uint32_t dst) {
    sg_command c{};
    c.type = SG_CMD_RESOLVE;
    c.texture = src;
    c.texture2 = dst;
    push(c, {});
  }
  // Submits the queue; the queries of its draws get their counters.
  int32_t flush() {
    if (cmds_.empty()) return pending_;
    bool counted = false;
    for (auto const& q : queries_) counted = counted || !q.empty();
    std::vector<sg_draw_stats> st(counted ? cmds_.size() : 0);
    int32_t r = sg_submit(dev, cmds_.data(), static_cast<uint32_t>(cmds_.size()), counted ? st.data() : nullptr);
    if (r == SG_OK && counted)
      for (size_t i = 0; i < cmds_.size(); ++i)
        for (auto const& q : queries_[i]) {
          q->ia_vertices += st[i].ia_vertices;
          q->ia_primitives += st[i].ia_primitives;
          q->vs_invocations += st[i].vs_invocations;
          q->cinvocations += st[i].cinvocations;
          q->cprimitives += st[i].cprimitives;
          q->ps_invocations += st[i].ps_invocations;
          q->backend_input_pixels += st[i].backend_input_pixels;
        }
    cmds_.clear();
    descs_.clear();
    queries_.clear();
    if (pending_ != SG_OK) r = pending_;
    pending_ = SG_OK;
    return r;
  }

private:
  void push(sg_command const& c, std::vector<std::shared_ptr<query_counters>> const& q) {
    cmds_.push_back(c);
    queries_.push_back(q);
    if (cmds_.size() >= max_queued) {
      int32_t r = flush();
      if (r != SG_OK) pending_ = r;  // reported by the next submitting call
    }
  }
  std::deque<sg_draw_desc> descs_;  // stable addresses for cmds_[i].draw
  std::vector<sg_command> cmds_;
  std::vector<std::vector<std::shared_ptr<query_counters>>> queries_;
  int32_t pending_ = SG_OK;
};
using device_sp = std::shared_ptr<device_ref>;
}  // namespace detail

}  // namespace salvia::core

namespace salvia::resource {

using salvia::core::color_rgba32f;

// A device buffer (buffer.h).  map/unmap go through a host copy.
class buffer {
public:
  buffer(core::detail::device_sp d, uint32_t h, size_t size) : dev_(std::move(d)), handle_(h), size_(size) {}
  ~buffer() {
    if (handle_) {
      dev_->flush();
      sg_buffer_destroy(dev_->dev, handle_);
    }
  }
  size_t size() const { return size_; }
  uint32_t handle() const { return handle_; }
  // buffer::transfer: copies host bytes into the buffer at `offset` (after
  // the queued commands that read it).
  result transfer(size_t offset, void const* src, size_t sz) {
    if (result r = to_result(dev_->flush()); r != result::ok) return r;
    return to_result(sg_buffer_upload(dev_->dev, handle_, offset, src, sz));
  }
  result read(size_t offset, void* dst, size_t sz) const {
    if (result r = to_result(dev_->flush()); r != result::ok) return r;
    return to_result(sg_buffer_download(dev_->dev, handle_, offset, dst, sz));
  }

private:
  core::detail::device_sp dev_;
  uint32_t handle_;
  size_t size_;
};
using buffer_ptr = std::shared_ptr<buffer>;

class texture;
// One mip level of a texture (surface.h); render targets name level 0.
class surface {
public:
  surface(std::shared_ptr<texture> const& tex, uint32_t level) : tex_(tex), level_(level) {}
  std::shared_ptr<texture> get_texture() const { return tex_.lock(); }
  uint32_t level() const { return level_; }
  size_t width() const;
  size_t height() const;
  size_t sample_count() const;
  pixel_format get_pixel_format() const;
  // bytes per row of texels (surface.h:48)
  size_t pitch() const { return width() * sample_count() * elem_size(); }
  // bytes per sample of the surface's format
  size_t elem_size() const;
  // Raw texels, layout ((y * w + x) * samples + s) * elem (surface.cpp:277-295).
  result read(std::vector<uint8_t>& out) const;
  result write(void const* data, size_t size);
  // surface::resolve (surface.cpp:123-140): box average of the samples into `target`.
  result resolve(surface& target);

private:
  std::weak_ptr<texture> tex_;
  uint32_t level_;
};
using surface_ptr = std::shared_ptr<surface>;

class texture : public std::enable_shared_from_this<texture> {
public:
  texture(core::detail::device_sp d, uint32_t h) : dev_(std::move(d)), handle_(h) {}
  ~texture() {
    if (handle_) {
      dev_->flush();
      sg_texture_destroy(dev_->dev, handle_);
    }
  }
  uint32_t handle() const { return handle_; }
  sg_device* device() const { return dev_->dev; }
  core::detail::device_ref& device_ref() const { return *dev_; }
  uint32_t levels() const {
    uint32_t n = 0;
    sg_texture_info(dev_->dev, handle_, 0, nullptr, nullptr, nullptr, nullptr, &n);
    return n;
  }
  // texture_cube::subresource(face, lod) (texture.h:97-99): lod * 6 + face
  surface_ptr subresource(size_t face, size_t lod) { return subresource(lod * 6 + face); }
  // texture::subresource (texture.h:17-80)
  surface_ptr subresource(size_t level) {
    if (level >= levels()) return nullptr;
    auto it = surfaces_.find(level);
    if (it != surfaces_.end()) return it->second;
    auto s = std::make_shared<surface>(shared_from_this(), static_cast<uint32_t>(level));
    surfaces_[level] = s;
    return s;
  }
  // texture::gen_mipmap(filter, auto_gen) (texture2d.cpp:25-36)
  result gen_mipmap(filter_type filter, bool /*auto_gen*/) {
    if (result r = to_result(dev_->flush()); r != result::ok) return r;
    surfaces_.clear();
    return to_result(sg_texture_gen_mipmap(dev_->dev, handle_, static_cast<uint32_t>(filter)));
  }
  size_t width(size_t level = 0) const { return info(level, 0); }
  size_t height(size_t level = 0) const { return info(level, 1); }
  size_t sample_count() const { return info(0, 2); }
  pixel_format get_pixel_format() const { return static_cast<pixel_format>(info(0, 3)); }

private:
  size_t info(size_t level, int what) const {
    uint32_t v[4] = {0, 0, 0, 0};
    sg_texture_info(dev_->dev, handle_, static_cast<uint32_t>(level), &v[0], &v[1], &v[2], &v[3], nullptr);
    return v[what];
  }
  core::detail::device_sp dev_;
  uint32_t handle_;
  std::map<size_t, surface_ptr> surfaces_;
};
using texture_ptr = std::shared_ptr<texture>;

inline size_t surface::width() const { return tex_.lock()->width(level_); }
inline size_t surface::height() const { return tex_.lock()->height(level_); }
inline size_t surface::sample_count() const { return tex_.lock()->sample_count(); }
inline pixel_format surface::get_pixel_format() const { return tex_.lock()->get_pixel_format(); }
inline size_t surface::elem_size() const {
  uint32_t const f = static_cast<uint32_t>(get_pixel_format());
  return f == SG_FMT_RGBA32F ? 16 : f == SG_FMT_RGB32F ? 12 : (f == SG_FMT_RG32F || f == SG_FMT_RGBA16F) ? 8 : 4;
}
inline result surface::read(std::vector<uint8_t>& out) const {
  auto t = tex_.lock();
  if (!t) return result::failed;
  if (result r = to_result(t->device_ref().flush()); r != result::ok) return r;
  uint32_t w = 0, h = 0, s = 0, f = 0;
  sg_texture_info(t->device(), t->handle(), level_, &w, &h, &s, &f, nullptr);
  out.resize(static_cast<size_t>(w) * h * s * elem_size());
  return to_result(sg_texture_download(t->device(), t->handle(), level_, out.data(), out.size()));
}
inline result surface::write(void const* data, size_t size) {
  auto t = tex_.lock();
  if (!t) return result::failed;
  if (result r = to_result(t->device_ref().flush()); r != result::ok) return r;
  return to_result(sg_texture_upload(t->device(), t->handle(), level_, data, size));
}
// Queued with the renderer's commands (it runs after the draws before it).
inline result surface::resolve(surface& target) {
  auto a = tex_.lock();
  auto b = target.tex_.lock();
  if (!a || !b || level_ != 0 || target.level_ != 0 || a.get() == b.get()) return result::invalid_parameter;
  if (b->sample_count() != 1 || a->width() != b->width() || a->height() != b->height()) return result::invalid_parameter;
  a->device_ref().queue_resolve(a->handle(), b->handle());
  return result::ok;
}

// sampler_desc (sampler.h:16-45)
struct sampler_desc {
  filter_type min_filter = filter_point;
  filter_type mag_filter = filter_point;
  filter_type mip_filter = filter_point;
  mip_quality mip_qual = mip_mi_quality;
  address_mode addr_mode_u = address_wrap;
  address_mode addr_mode_v = address_wrap;
  address_mode addr_mode_w = address_wrap;
  float mip_lod_bias = 0;
  uint32_t max_anisotropy = 0;
  compare_function comparison_func = compare_function_always;
  color_rgba32f border_color{0, 0, 0, 0};
  float min_lod = -1e20f;
  float max_lod = 1e20f;
};

class sampler {
public:
  sampler(core::detail::device_sp d, uint32_t h, sampler_desc const& desc, texture_ptr tex)
      : dev_(std::move(d)), handle_(h), desc_(desc), tex_(std::move(tex)) {}
  ~sampler() {
    if (handle_) {
      dev_->flush();  // queued draws may sample through it
      sg_sampler_destroy(dev_->dev, handle_);
    }
  }
  uint32_t handle() const { return handle_; }
  sampler_desc const& get_desc() const { return desc_; }
  texture_ptr const& get_texture() const { return tex_; }

private:
  core::detail::device_sp dev_;
  uint32_t handle_;
  sampler_desc desc_;
  texture_ptr tex_;
};
using sampler_ptr = std::shared_ptr<sampler>;

enum input_classifications { input_per_vertex };

// input_element_desc (input_layout.h:20-47)
struct input_element_desc {
  std::string semantic_name;
  uint32_t semantic_index = 0;
  format data_format = format_unknown;
  uint32_t input_slot = 0;
  uint32_t aligned_byte_offset = 0xFFFFFFFFu;
  input_classifications slot_class = input_per_vertex;
  uint32_t instance_data_step_rate = 0;
  input_element_desc() = default;
  input_element_desc(char const* name, uint32_t index, format fmt, uint32_t slot, uint32_t offset,
                     input_classifications cls, uint32_t step)
      : semantic_name(name), semantic_index(index), data_format(fmt), input_slot(slot),
        aligned_byte_offset(offset), slot_class(cls), instance_data_step_rate(step) {}
};

// The elements bound to vertex-shader input registers (renderer::create_input_layout
// with a cpp_vertex_shader, renderer_impl.cpp; stream_assembler.cpp:26-93).
class input_layout {
public:
  std::vector<sg_vs_input> registers;
};
using input_layout_ptr = std::shared_ptr<input_layout>;

}  // namespace salvia::resource

namespace salvia::core {

using resource::buffer_ptr;
using resource::input_element_desc;
using resource::input_layout_ptr;
using resource::sampler_desc;
using resource::sampler_ptr;
using resource::surface_ptr;
using resource::texture_ptr;

// raster_desc / raster_state (raster_state.h:17-68)
struct raster_desc {
  fill_mode fm = fill_solid;
  cull_mode cm = cull_back;
  bool front_ccw = false;
  int32_t depth_bias = 0;
  float depth_bias_clamp = 0;
  float slope_scaled_depth_bias = 0;
  bool depth_clip_enable = true;
  bool scissor_enable = false;
  bool multisample_enable = true;
  bool anti_aliased_line_enable = false;
};
class raster_state {
public:
  explicit raster_state(raster_desc const& d) : desc_(d) {}
  raster_desc const& get_desc() const { return desc_; }

private:
  raster_desc desc_;
};
using raster_state_ptr = std::shared_ptr<raster_state>;

// depth_stencil_desc / depth_stencil_state (framebuffer.h:20-77)
struct depth_stencil_op_desc {
  stencil_op stencil_fail_op = stencil_op_keep;
  stencil_op stencil_depth_fail_op = stencil_op_keep;
  stencil_op stencil_pass_op = stencil_op_keep;
  compare_function stencil_func = compare_function_always;
};
struct depth_stencil_desc {
  bool depth_enable = true;
  bool depth_write_mask = true;
  compare_function depth_func = compare_function_less;
  bool stencil_enable = false;
  uint8_t stencil_read_mask = 0xFF;
  uint8_t stencil_write_mask = 0xFF;
  depth_stencil_op_desc front_face;
  depth_stencil_op_desc back_face;
};
class depth_stencil_state {
public:
  explicit depth_stencil_state(depth_stencil_desc const& d) : desc_(d) {}
  depth_stencil_desc const& get_desc() const { return desc_; }

private:
  depth_stencil_desc desc_;
};
using depth_stencil_state_ptr = std::shared_ptr<depth_stencil_state>;

// ---- shaders ------------------------------------------------------------
namespace am {  // vs_output::attrib_modifier_type (shader_regs.h:49-55)
enum { am_linear = SG_AM_LINEAR, am_centroid = SG_AM_CENTROID, am_nointerpolation = SG_AM_NOINTERPOLATION,
       am_noperspective = SG_AM_NOPERSPECTIVE, am_sample = SG_AM_SAMPLE };
}

class cpp_shader;
using cpp_shader_ptr = std::shared_ptr<cpp_shader>;

class cpp_shader {
public:
  virtual ~cpp_shader() = default;
  virtual result set_sampler(std::string const& name, sampler_ptr const& samp) = 0;
  virtual result set_constant(std::string const& name, void const* pval) = 0;
  virtual cpp_shader_ptr clone() = 0;
  // The device program this shader runs (SG_VS_* / SG_PS_* / SG_BS_*).
  virtual uint32_t program() const = 0;
  // The learned filter an SG_PS_TEX_GRAD_LEARNED program uses (sg_af_model_id), else 0.
  virtual uint32_t learned_filter() const { return 0; }
};

// cpp_shader_impl (shader.h:86-157): named constants and samplers, and the
// semantic -> input-register map of a vertex shader.  Constants are packed,
// in declaration order, into the program's float constant block; samplers,
// in declaration order, into its sampler slots.
class cpp_shader_impl : public cpp_shader {
public:
  result set_sampler(std::string const& name, sampler_ptr const& samp) override {
    for (auto& s : samplers_)
      if (s.first == name) {
        *s.second = samp;
        return result::ok;
      }
    return result::failed;
  }
  result set_constant(std::string const& name, void const* pval) override {
    for (auto& c : constants_)
      if (c.name == name) {
        std::memcpy(c.ptr, pval, c.size);
        return result::ok;
      }
    return result::failed;
  }
  template <class T>
  result declare_constant(std::string const& name, T& var) {
    static_assert(sizeof(T) % 4 == 0, "shader constants are packed as 32-bit words");
    constants_.push_back({name, &var, sizeof(T)});
    return result::ok;
  }
  result declare_sampler(std::string const& name, sampler_ptr& var) {
    samplers_.push_back({name, &var});
    return result::ok;
  }
  void bind_semantic(char const* name, size_t semantic_index, size_t register_index) {
    regs_[std::string(name) + "#" + std::to_string(semantic_index)] = register_index;
  }
  result find_register(char const* name, size_t semantic_index, size_t& index) const {
    auto it = regs_.find(std::string(name) + "#" + std::to_string(semantic_index));
    if (it == regs_.end()) return result::failed;
    index = it->second;
    return result::ok;
  }
  // Fills `s` with the program, constants and samplers of this shader.
  result pack(sg_shader& s) const {
    std::memset(&s, 0, sizeof(s));
    s.program = program();
    s.learned_filter = learned_filter();
    size_t off = 0;
    for (auto const& c : constants_) {
      size_t n = c.size / 4;
      if (off + n > SG_MAX_SHADER_CONSTANTS) return result::invalid_parameter;
      std::memcpy(&s.constants[off], c.ptr, c.size);
      off += n;
    }
    if (samplers_.size() > SG_MAX_SHADER_SAMPLERS) return result::invalid_parameter;
    for (size_t i = 0; i < samplers_.size(); ++i) s.samplers[i] = *samplers_[i].second ? (*samplers_[i].second)->handle() : 0;
    return result::ok;
  }
  std::unordered_map<std::string, size_t> const& register_map() const { return regs_; }

  cpp_shader_impl() = default;
  // Copies re-point the declared constants and samplers at the copy's members
  // (the offsets of the declared members within the object are kept).
  cpp_shader_impl(cpp_shader_impl const& o) : regs_(o.regs_) { rebase(o); }
  cpp_shader_impl& operator=(cpp_shader_impl const& o) {
    regs_ = o.regs_;
    rebase(o);
    return *this;
  }

private:
  struct constant {
    std::string name;
    void* ptr;
    size_t size;
  };
  void rebase(cpp_shader_impl const& o) {
    auto const* ob = reinterpret_cast<char const*>(&o);
    auto* nb = reinterpret_cast<char*>(this);
    constants_.clear();
    samplers_.clear();
    for (auto const& c : o.constants_)
      constants_.push_back({c.name, nb + (static_cast<char const*>(c.ptr) - ob), c.size});
    for (auto const& s : o.samplers_)
      samplers_.push_back({s.first, reinterpret_cast<sampler_ptr*>(nb + (reinterpret_cast<char const*>(s.second) - ob))});
  }
  std::vector<constant> constants_;
  std::vector<std::pair<std::string, sampler_ptr*>> samplers_;
  std::unordered_map<std::string, size_t> regs_;
};

// cpp_vertex_shader (shader.h:159-165)
class cpp_vertex_shader : public cpp_shader_impl {
public:
  virtual uint32_t num_output_attributes() const = 0;
  virtual uint32_t output_attribute_modifiers(uint32_t index) const = 0;
};
// cpp_pixel_shader (shader.h:169-205)
class cpp_pixel_shader : public cpp_shader_impl {};
// cpp_blend_shader (shader.h:209-215)
class cpp_blend_shader : public cpp_shader_impl {};

using cpp_vertex_shader_ptr = std::shared_ptr<cpp_vertex_shader>;
using cpp_pixel_shader_ptr = std::shared_ptr<cpp_pixel_shader>;
using cpp_blend_shader_ptr = std::shared_ptr<cpp_blend_shader>;

#define SALVIA_GB300_CLONE(cls) \
  cpp_shader_ptr clone() override { return cpp_shader_ptr(new cls(*this)); }

// ---- stock shaders: the device programs the library ships ---------------
// out.position = transform(in[0], WorldViewProjMat); out.attr[i] = in[i + 1].
class transform_vertex_shader : public cpp_vertex_shader {
public:
  explicit transform_vertex_shader(uint32_t num_attributes, mat44 const& m = mat44::identity(),
                                   uint32_t modifiers = am::am_linear)
      : wvp_(m), nattr_(num_attributes), mods_(modifiers) {
    declare_constant("WorldViewProjMat", wvp_);
  }
  uint32_t program() const override { return SG_VS_TRANSFORM; }
  uint32_t num_output_attributes() const override { return nattr_; }
  uint32_t output_attribute_modifiers(uint32_t) const override { return mods_; }
  SALVIA_GB300_CLONE(transform_vertex_shader)

private:
  mat44 wvp_;
  uint32_t nattr_, mods_;
};
// out.color[0] = in.attr[0]
// out.color[i] = in.attr[i]: one colour per bound target (SG_PS_COLOR_MRT).
class color_mrt_pixel_shader : public cpp_pixel_shader {
public:
  uint32_t program() const override { return SG_PS_COLOR_MRT; }
  SALVIA_GB300_CLONE(color_mrt_pixel_shader)
};
class color_pixel_shader : public cpp_pixel_shader {
public:
  uint32_t program() const override { return SG_PS_COLOR; }
  SALVIA_GB300_CLONE(color_pixel_shader)
};
// out.color[0] = Color
class constant_pixel_shader : public cpp_pixel_shader {
public:
  explicit constant_pixel_shader(vec4 const& c = vec4{}) : color_(c) { declare_constant("Color", color_); }
  uint32_t program() const override { return SG_PS_CONSTANT; }
  SALVIA_GB300_CLONE(constant_pixel_shader)

private:
  vec4 color_;
};
// out.color[0] = tex2d(Sampler, 0) * in.attr[1]
class texture_pixel_shader : public cpp_pixel_shader {
public:
  explicit texture_pixel_shader(sampler_ptr const& s = nullptr) : samp_(s) { declare_sampler("Sampler", samp_); }
  uint32_t program() const override { return SG_PS_TEX_MODULATE; }
  SALVIA_GB300_CLONE(texture_pixel_shader)

private:
  sampler_ptr samp_;
};
// out.color[0] = Sampler.sample_2d_grad(in.attr[0].xy, ddx(0), ddy(0), 0) * in.attr[1]
class texture_grad_pixel_shader : public cpp_pixel_shader {
public:
  explicit texture_grad_pixel_shader(sampler_ptr const& s = nullptr) : samp_(s) { declare_sampler("Sampler", samp_); }
  uint32_t program() const override { return SG_PS_TEX_GRAD_MODULATE; }
  SALVIA_GB300_CLONE(texture_grad_pixel_shader)

private:
  sampler_ptr samp_;
};
// tex2dlod(Sampler, 0) * in.attr[1]: the level is attr[0].w (cpp_pixel_shader.cpp:33-40).
class texture_lod_pixel_shader : public cpp_pixel_shader {
public:
  explicit texture_lod_pixel_shader(sampler_ptr const& s = nullptr) : samp_(s) { declare_sampler("Sampler", samp_); }
  uint32_t program() const override { return SG_PS_TEX_LOD_MODULATE; }
  SALVIA_GB300_CLONE(texture_lod_pixel_shader)

private:
  sampler_ptr samp_;
};
// tex2dproj(Sampler, 0) * in.attr[1] (cpp_pixel_shader.cpp:42-60).
class texture_proj_pixel_shader : public cpp_pixel_shader {
public:
  explicit texture_proj_pixel_shader(sampler_ptr const& s = nullptr) : samp_(s) { declare_sampler("Sampler", samp_); }
  uint32_t program() const override { return SG_PS_TEX_PROJ_MODULATE; }
  SALVIA_GB300_CLONE(texture_proj_pixel_shader)

private:
  sampler_ptr samp_;
};
// Alpha test: tex2d(Sampler, 0) * in.attr[1], discarded below the "AlphaRef" alpha.
class alpha_test_pixel_shader : public cpp_pixel_shader {
public:
  explicit alpha_test_pixel_shader(float alpha_ref = 0.5f, sampler_ptr const& s = nullptr) : ref_(alpha_ref), samp_(s) {
    declare_constant("AlphaRef", ref_);
    declare_sampler("Sampler", samp_);
  }
  uint32_t program() const override { return SG_PS_TEX_ALPHA_TEST; }
  SALVIA_GB300_CLONE(alpha_test_pixel_shader)

private:
  float ref_;
  sampler_ptr samp_;
};
// No counterpart in the reference: texture_grad_pixel_shader with the
// anisotropic lookup on a learned filter (SG_PS_TEX_GRAD_LEARNED) where its
// probe count lies in (MinProbes, MaxProbes] and its confidence reaches
// ConfidenceThreshold; the plain sampler everywhere else.
class learned_texture_grad_pixel_shader : public cpp_pixel_shader {
public:
  learned_texture_grad_pixel_shader(sampler_ptr const& s, uint32_t filter_id, float confidence_threshold = 0.5f,
                                    float max_probes = 16.0f, float min_probes = 0.0f)
      : samp_(s), filter_(filter_id), thr_(confidence_threshold), max_(max_probes), min_(min_probes) {
    declare_sampler("Sampler", samp_);
    declare_constant("ConfidenceThreshold", thr_);
    declare_constant("MaxProbes", max_);
    declare_constant("MinProbes", min_);
  }
  uint32_t program() const override { return SG_PS_TEX_GRAD_LEARNED; }
  uint32_t learned_filter() const override { return filter_; }
  SALVIA_GB300_CLONE(learned_texture_grad_pixel_shader)

private:
  sampler_ptr samp_;
  uint32_t filter_;
  float thr_, max_, min_;
};
// A user pixel or blend shader (a registered module's program id); its
// constants and sampler are declared by a subclass as for any cpp shader.
// A registered user vertex shader module (SALVIA_GB300_VERTEX_SHADER): the
// application declares its constants (up to SG_MAX_SHADER_CONSTANTS floats,
// in declaration order) and its sampler like any cpp_vertex_shader.
class module_vertex_shader : public cpp_vertex_shader {
public:
  module_vertex_shader(uint32_t program_id, uint32_t num_attributes, uint32_t modifiers = am::am_linear)
      : prog_(program_id), nattr_(num_attributes), mods_(modifiers) {}
  uint32_t program() const override { return prog_; }
  uint32_t num_output_attributes() const override { return nattr_; }
  uint32_t output_attribute_modifiers(uint32_t) const override { return mods_; }
  SALVIA_GB300_CLONE(module_vertex_shader)

private:
  uint32_t prog_, nattr_, mods_;
};
class module_pixel_shader : public cpp_pixel_shader {
public:
  explicit module_pixel_shader(uint32_t program_id) : prog_(program_id) {}
  uint32_t program() const override { return prog_; }
  SALVIA_GB300_CLONE(module_pixel_shader)

private:
  uint32_t prog_;
};
class module_blend_shader : public cpp_blend_shader {
public:
  explicit module_blend_shader(uint32_t program_id) : prog_(program_id) {}
  uint32_t program() const override { return prog_; }
  SALVIA_GB300_CLONE(module_blend_shader)

private:
  uint32_t prog_;
};
class replace_blend_shader : public cpp_blend_shader {  // color(0, s) = src
public:
  uint32_t program() const override { return SG_BS_REPLACE; }
  SALVIA_GB300_CLONE(replace_blend_shader)
};
class src_alpha_blend_shader : public cpp_blend_shader {  // lerp(dst, src, src.a)
public:
  uint32_t program() const override { return SG_BS_LERP_SRC_ALPHA; }
  SALVIA_GB300_CLONE(src_alpha_blend_shader)
};
class replace_all_blend_shader : public cpp_blend_shader {  // color(i, s) = in.color[i], every target
public:
  uint32_t program() const override { return SG_BS_REPLACE_ALL; }
  SALVIA_GB300_CLONE(replace_all_blend_shader)
};
class additive_blend_shader : public cpp_blend_shader {  // dst + src
public:
  uint32_t program() const override { return SG_BS_ADD; }
  SALVIA_GB300_CLONE(additive_blend_shader)
};

// ---- queries (async_object.h:90-233) ------------------------------------
struct pipeline_statistics {
  uint64_t ia_vertices, ia_primitives, vs_invocations, gs_invocations, gs_primitives, cinvocations, cprimitives,
      ps_invocations;
};
struct internal_statistics {
  uint64_t backend_input_pixels;
};
class async_object {
public:
  explicit async_object(async_object_ids id) : id_(id) {}
  async_object_ids id() const { return id_; }
  bool running = false;
  // added up by the queued draws issued while the query runs
  std::shared_ptr<detail::query_counters> counters = std::make_shared<detail::query_counters>();

private:
  async_object_ids id_;
};
using async_object_ptr = std::shared_ptr<async_object>;

struct mapped_resource {
  void* data = nullptr;
  size_t row_pitch = 0, depth_pitch = 0;
};

// ---- the renderer (renderer.h:42-131) -----------------------------------
// No counterpart in the reference: a learned anisotropic filter (sg_af_model)
// owned by a renderer's device.  Train it on the device from the plain
// sampler, then hand id() to learned_texture_grad_pixel_shader.
class learned_filter {
public:
  learned_filter(detail::device_sp d, sg_af_model* m) : dev_(std::move(d)), model_(m) {}
  ~learned_filter() {
    if (model_) sg_af_model_destroy(dev_->dev, model_);
  }
  learned_filter(learned_filter const&) = delete;
  learned_filter& operator=(learned_filter const&) = delete;
  uint32_t id() const { return sg_af_model_id(model_); }
  sg_af_model* native() const { return model_; }
  // Trains on lookups of the plain anisotropic sampler over the samplers'
  // textures (sg_af_model_train).
  result train(std::vector<sampler_ptr> const& samplers, uint32_t samples, uint32_t batch = 8192, uint32_t epochs = 2,
               float lr = 2e-3f, uint64_t seed = 1, sg_af_report* report = nullptr) {
    std::vector<uint32_t> h;
    for (auto const& sp : samplers) h.push_back(sp ? sp->handle() : 0u);
    sg_af_train_desc t{};
    t.samplers = h.data();
    t.num_samplers = static_cast<uint32_t>(h.size());
    t.samples = samples;
    t.batch = batch;
    t.epochs = epochs;
    t.lr = lr;
    t.seed = seed;
    return to_result(sg_af_model_train(dev_->dev, model_, &t, report));
  }

private:
  detail::device_sp dev_;
  sg_af_model* model_ = nullptr;
};
using learned_filter_ptr = std::shared_ptr<learned_filter>;

class renderer {
public:
  explicit renderer(sg_device* d) : dev_(std::make_shared<detail::device_ref>(d)) {
    vp_ = viewport{0, 0, 0, 0, 0, 1};
    rs_ = std::make_shared<raster_state>(raster_desc{});
    dss_ = std::make_shared<depth_stencil_state>(depth_stencil_desc{});
  }
  sg_device* native() const { return dev_->dev; }
  char const* last_error() const { return sg_last_error(dev_->dev); }

  // creators
  buffer_ptr create_buffer(size_t size) {
    uint32_t h = 0;
    if (sg_buffer_create(dev_->dev, size, &h) != SG_OK) return nullptr;
    return std::make_shared<resource::buffer>(dev_, h, size);
  }
  texture_ptr create_tex2d(size_t width, size_t height, size_t num_samples, pixel_format fmt) {
    uint32_t h = 0;
    if (sg_texture_create(dev_->dev, static_cast<uint32_t>(width), static_cast<uint32_t>(height),
                          static_cast<uint32_t>(num_samples), static_cast<uint32_t>(fmt), &h) != SG_OK)
      return nullptr;
    return std::make_shared<resource::texture>(dev_, h);
  }
  sampler_ptr create_sampler(sampler_desc const& desc, texture_ptr const& tex) {
    if (!tex) return nullptr;
    sg_sampler_desc d{};
    d.min_filter = desc.min_filter;
    d.mag_filter = desc.mag_filter;
    d.mip_filter = desc.mip_filter;
    d.mip_quality = desc.mip_qual;
    d.address_u = desc.addr_mode_u;
    d.address_v = desc.addr_mode_v;
    d.address_w = desc.addr_mode_w;
    d.max_anisotropy = desc.max_anisotropy;
    d.lod_bias = desc.mip_lod_bias;
    d.border_color[0] = desc.border_color.r;
    d.border_color[1] = desc.border_color.g;
    d.border_color[2] = desc.border_color.b;
    d.border_color[3] = desc.border_color.a;
    d.min_lod = desc.min_lod;
    d.max_lod = desc.max_lod;
    uint32_t h = 0;
    if (sg_sampler_create(dev_->dev, &d, tex->handle(), &h) != SG_OK) return nullptr;
    return std::make_shared<resource::sampler>(dev_, h, desc, tex);
  }
  // No counterpart in the reference: a learned anisotropic filter on this
  // renderer's device (sg_af_model_create), untrained.
  learned_filter_ptr create_learned_filter(uint64_t seed = 1) {
    sg_af_model* m = nullptr;
    if (sg_af_model_create(dev_->dev, seed, &m) != SG_OK) return nullptr;
    return std::make_shared<learned_filter>(dev_, m);
  }
  // No counterpart in the reference: makes a user shader module
  // (salvia_gb300/device_shader.cuh) a program of this renderer's device; a
  // cpp_pixel_shader / cpp_blend_shader subclass returns the id from
  // program() (module_vertex_shader / module_pixel_shader /
  // module_blend_shader do).  0 on failure.
  uint32_t register_shader(sg_shader_module const* m) {
    uint32_t id = 0;
    return sg_shader_register(dev_->dev, m, &id) == SG_OK ? id : 0u;
  }
  // renderer::create_texcube (renderer.h:49): six faces, subresource(face)
  // in cubemap_faces order; a cube's LOD range stays [0, 0] as in the reference.
  texture_ptr create_texcube(size_t width, size_t height, size_t num_samples, pixel_format fmt) {
    uint32_t h = 0;
    if (sg_texture_create_cube(dev_->dev, static_cast<uint32_t>(width), static_cast<uint32_t>(height),
                               static_cast<uint32_t>(num_samples), static_cast<uint32_t>(fmt), &h) != SG_OK)
      return nullptr;
    return std::make_shared<resource::texture>(dev_, h);
  }
  async_object_ptr create_query(async_object_ids id) {
    if (id != async_object_ids::pipeline_statistics && id != async_object_ids::internal_statistics) return nullptr;
    return std::make_shared<async_object>(id);
  }
  // The SASL overload (renderer.h:52-54): the elements bound to the
  // compiled vertex shader's input registers by semantic.
  input_layout_ptr create_input_layout(input_element_desc const* descs, size_t count,
                                       shader::shader_object_ptr const& vs) {
    if (!vs || vs->language != shader::lang_vertex_shader) return nullptr;
    return make_layout(descs, count, [&](std::string const& name, size_t index, size_t& reg) {
      for (auto const& in : vs->inputs)
        if (salvia::detail::same_semantic(in.semantic, name) && in.index == index) {
          reg = static_cast<size_t>(in.reg);
          return true;
        }
      return false;
    });
  }
  // Binds the elements to the shader's input registers by semantic
  // (renderer::create_input_layout(descs, n, cpp_vertex_shader_ptr)).
  input_layout_ptr create_input_layout(input_element_desc const* descs, size_t count, cpp_vertex_shader_ptr const& vs) {
    if (!vs) return nullptr;
    return make_layout(descs, count, [&](std::string const& name, size_t index, size_t& reg) {
      return vs->find_register(name.c_str(), index, reg) == result::ok;
    });
  }

private:
  input_layout_ptr make_layout(input_element_desc const* descs, size_t count,
                               std::function<bool(std::string const&, size_t, size_t&)> const& find) {
    auto il = std::make_shared<resource::input_layout>();
    for (size_t i = 0; i < count; ++i) {
      size_t reg = 0;
      if (!find(descs[i].semantic_name, descs[i].semantic_index, reg)) continue;
      if (reg >= SG_MAX_VS_INPUTS) return nullptr;
      if (il->registers.size() <= reg) il->registers.resize(reg + 1, sg_vs_input{SG_SEMANTIC_TEXCOORD, 0,
                                                                                  SG_VFMT_R32G32B32A32_FLOAT, 0, 0});
      sg_vs_input& r = il->registers[reg];
      std::string const& n = descs[i].semantic_name;
      r.semantic = n == "POSITION" || n == "SV_Position" ? SG_SEMANTIC_POSITION
                   : n == "COLOR" ? SG_SEMANTIC_COLOR : n == "NORMAL" ? SG_SEMANTIC_NORMAL : SG_SEMANTIC_TEXCOORD;
      r.semantic_index = descs[i].semantic_index;
      r.format = descs[i].data_format;
      r.slot = descs[i].input_slot;
      r.offset = descs[i].aligned_byte_offset == 0xFFFFFFFFu ? 0 : descs[i].aligned_byte_offset;
    }
    return il;
  }

public:

  // map / unmap (renderer.h:61-63): a host copy, written back on unmap.
  result map(mapped_resource& mr, buffer_ptr const& buf, map_mode mm) {
    if (!buf || mapped_buf_ || mapped_surf_) return result::failed;
    shadow_.assign(buf->size(), 0);
    if (mm == map_read || mm == map_read_write || mm == map_write_no_overwrite)
      if (buf->read(0, shadow_.data(), shadow_.size()) != result::ok) return result::failed;
    mapped_buf_ = buf;
    mapped_mode_ = mm;
    mr.data = shadow_.data();
    mr.row_pitch = mr.depth_pitch = buf->size();
    return result::ok;
  }
  // A surface maps as its texels, ((y * w + x) * samples + s) * elem, with
  // the row and slice pitches of surface::map (surface.cpp:94-116).
  result map(mapped_resource& mr, surface_ptr const& surf, map_mode mm) {
    if (!surf || mapped_buf_ || mapped_surf_ || !surf->height()) return result::failed;
    if (surf->read(shadow_) != result::ok) return result::failed;
    mapped_surf_ = surf;
    mapped_mode_ = mm;
    mr.data = shadow_.data();
    mr.row_pitch = shadow_.size() / surf->height();
    mr.depth_pitch = shadow_.size();
    return result::ok;
  }
  result unmap() {
    if (!mapped_buf_ && !mapped_surf_) return result::failed;
    result r = result::ok;
    if (mapped_buf_ && mapped_mode_ != map_read) r = mapped_buf_->transfer(0, shadow_.data(), shadow_.size());
    if (mapped_surf_ && mapped_mode_ != map_read) r = mapped_surf_->write(shadow_.data(), shadow_.size());
    mapped_buf_.reset();
    mapped_surf_.reset();
    return r;
  }

  // state set
  result set_vertex_buffers(size_t start_slot, size_t count, buffer_ptr const* buffers, size_t const* strides,
                            size_t const* offsets) {
    if (start_slot + count > SG_MAX_STREAMS) return result::invalid_parameter;
    for (size_t i = 0; i < count; ++i) {
      streams_[start_slot + i] = buffers[i];
      strides_[start_slot + i] = strides[i];
      offsets_[start_slot + i] = offsets[i];
    }
    return result::ok;
  }
  result set_index_buffer(buffer_ptr const& b, format fmt) {
    if (fmt != format_r16_uint && fmt != format_r32_uint) return result::invalid_parameter;
    ib_ = b;
    ib_fmt_ = fmt;
    return result::ok;
  }
  result set_input_layout(input_layout_ptr const& l) {
    layout_ = l;
    return result::ok;
  }
  result set_vertex_shader(cpp_vertex_shader_ptr const& vs) {
    vs_ = vs;
    return result::ok;
  }
  result set_pixel_shader(cpp_pixel_shader_ptr const& ps) {
    ps_ = ps;
    return result::ok;
  }
  result set_blend_shader(cpp_blend_shader_ptr const& bs) {
    bs_ = bs;
    return result::ok;
  }
  result set_primitive_topology(primitive_topology t) {
    topo_ = t;
    return result::ok;
  }
  result set_rasterizer_state(raster_state_ptr const& rs) {
    rs_ = rs ? rs : std::make_shared<raster_state>(raster_desc{});
    return result::ok;
  }
  result set_depth_stencil_state(depth_stencil_state_ptr const& dss, int32_t stencil_ref) {
    dss_ = dss ? dss : std::make_shared<depth_stencil_state>(depth_stencil_desc{});
    stencil_ref_ = stencil_ref;
    return result::ok;
  }
  // renderer_impl::set_render_targets (renderer_impl.cpp:159-238): fewer
  // than MAX_RENDER_TARGETS colour targets of one sample count, level-0
  // surfaces here; the depth-stencil target covers the smallest of them.
  result set_render_targets(size_t color_count, surface_ptr const* colors, surface_ptr const& ds) {
    colors_.clear();
    ds_.reset();
    if (color_count > SG_MAX_COLOR_TARGETS) return result::failed;
    if ((color_count == 0 || colors == nullptr) && !ds) return result::failed;
    size_t samples = 0, w = static_cast<size_t>(-1), h = static_cast<size_t>(-1);
    for (size_t i = 0; i < color_count && colors; ++i) {
      if (!colors[i] || colors[i]->level() != 0) return result::failed;
      if (samples == 0) samples = colors[i]->sample_count();
      if (colors[i]->sample_count() != samples) return result::failed;
      w = std::min(w, colors[i]->width());
      h = std::min(h, colors[i]->height());
    }
    if (ds && color_count && (ds->sample_count() != samples || ds->width() < w || ds->height() < h))
      return result::failed;
    if (colors) colors_.assign(colors, colors + color_count);
    ds_ = ds;
    return result::ok;
  }
  result set_viewport(viewport const& vp) {
    vp_ = vp;
    return result::ok;
  }
  // Shader-code state (renderer.h:75-101, renderer_impl.cpp:287-335): a
  // compiled SASL shader replaces the stage's cpp shader while it is set
  // (null clears it) and reads the variables and samplers set by name.
  result set_vertex_shader_code(shader::shader_object_ptr const& s) {
    if (s && (s->language != shader::lang_vertex_shader || !s->module)) return result::failed;
    vs_code_ = s;
    return result::ok;
  }
  result set_pixel_shader_code(shader::shader_object_ptr const& s) {
    if (s && (s->language != shader::lang_pixel_shader || !s->module)) return result::failed;
    ps_code_ = s;
    return result::ok;
  }
  result set_vs_variable_value(std::string const& name, void const* data, size_t sz) {
    return keep(vs_vars_, name, data, sz);
  }
  result set_vs_variable_pointer(std::string const& name, void const* data, size_t sz) {
    return keep(vs_vars_, name, data, sz);
  }
  template <typename T>
  result set_vs_variable(std::string const& name, T const* data) {
    return set_vs_variable_value(name, static_cast<void const*>(data), sizeof(T));
  }
  result set_ps_variable(std::string const& name, void const* data, size_t sz) { return keep(ps_vars_, name, data, sz); }
  template <typename T>
  result set_ps_variable(std::string const& name, T const* data) {
    return set_ps_variable(name, static_cast<void const*>(data), sizeof(T));
  }
  result set_vs_sampler(std::string const& name, sampler_ptr const& samp) {
    vs_samplers_[name] = samp;
    return result::ok;
  }
  result set_ps_sampler(std::string const& name, sampler_ptr const& samp) {
    ps_samplers_[name] = samp;
    return result::ok;
  }

  // state get
  buffer_ptr get_index_buffer() const { return ib_; }
  format get_index_format() const { return ib_fmt_; }
  primitive_topology get_primitive_topology() const { return topo_; }
  cpp_vertex_shader_ptr get_vertex_shader() const { return vs_; }
  raster_state_ptr get_rasterizer_state() const { return rs_; }
  cpp_pixel_shader_ptr get_pixel_shader() const { return ps_; }
  cpp_blend_shader_ptr get_blend_shader() const { return bs_; }
  viewport get_viewport() const { return vp_; }
  shader::shader_object_ptr get_vertex_shader_code() const { return vs_code_; }
  shader::shader_object_ptr get_pixel_shader_code() const { return ps_code_; }

  // queries
  result begin(async_object_ptr const& q) {
    if (!q || q->running) return result::failed;
    q->running = true;
    q->counters = std::make_shared<detail::query_counters>();  // draws still queued keep the old one
    queries_.push_back(q);
    return result::ok;
  }
  result end(async_object_ptr const& q) {
    if (!q || !q->running) return result::failed;
    q->running = false;
    for (size_t i = 0; i < queries_.size(); ++i)
      if (queries_[i] == q) {
        queries_.erase(queries_.begin() + static_cast<long>(i));
        break;
      }
    return result::ok;
  }
  // Submits the queued commands a query counts and waits for them.
  async_status get_data(async_object_ptr const& q, void* data, bool /*do_not_wait*/) {
    if (!q || q->running) return async_status::error;
    if (dev_->flush() != SG_OK || sg_sync(dev_->dev) != SG_OK) return async_status::error;
    detail::query_counters const& c = *q->counters;
    if (q->id() == async_object_ids::pipeline_statistics) {
      pipeline_statistics s{};
      s.ia_vertices = c.ia_vertices;
      s.ia_primitives = c.ia_primitives;
      s.vs_invocations = c.vs_invocations;
      s.cinvocations = c.cinvocations;
      s.cprimitives = c.cprimitives;
      s.ps_invocations = c.ps_invocations;
      std::memcpy(data, &s, sizeof(s));
    } else {
      internal_statistics s{c.backend_input_pixels};
      std::memcpy(data, &s, sizeof(s));
    }
    return async_status::ready;
  }

  // render operations: queued (see detail::device_ref), submitted together
  result draw(size_t startpos, size_t primcnt) { return submit(false, startpos, primcnt, 0); }
  result draw_index(size_t startpos, size_t primcnt, int basevert) { return submit(true, startpos, primcnt, basevert); }
  result clear_color(surface_ptr const& s, color_rgba32f const& c) {
    if (!s || s->level() != 0) return result::invalid_parameter;
    float rgba[4] = {c.r, c.g, c.b, c.a};
    dev_->queue_clear_color(s->get_texture()->handle(), rgba);
    return result::ok;
  }
  result clear_depth_stencil(surface_ptr const& s, uint32_t flags, float d, uint32_t st) {
    if (!s || s->level() != 0) return result::invalid_parameter;
    if (flags == 0 || flags > (clear_depth | clear_stencil)) return result::invalid_parameter;
    dev_->queue_clear_depth_stencil(s->get_texture()->handle(), flags, d, st);
    return result::ok;
  }
  // renderer::flush (renderer.h:128): submits the queued commands and waits for them
  result flush() {
    int32_t r = dev_->flush();
    int32_t s = sg_sync(dev_->dev);
    return to_result(r != SG_OK ? r : s);
  }

  // The C-ABI descriptor of a draw under the current state.
  result build_desc(bool indexed, size_t startpos, size_t primcnt, int basevert, sg_draw_desc& d) const {
    std::memset(&d, 0, sizeof(d));
    if ((!vs_ && !vs_code_) || (!ps_ && !ps_code_) || !bs_ || !layout_) return result::failed;
    d.color_target = colors_.empty() ? 0 : colors_[0]->get_texture()->handle();
    for (size_t i = 1; i < colors_.size(); ++i) d.more_color_targets[i - 1] = colors_[i]->get_texture()->handle();
    d.ds_target = ds_ ? ds_->get_texture()->handle() : 0;
    d.viewport = sg_viewport{vp_.x, vp_.y, vp_.w, vp_.h, vp_.minz, vp_.maxz};
    d.topology = topo_;
    d.indexed = indexed ? 1u : 0u;
    if (indexed) {
      if (!ib_) return result::failed;
      d.index_buffer = ib_->handle();
      d.index_format = ib_fmt_ == format_r16_uint ? SG_INDEX_U16 : SG_INDEX_U32;
    }
    d.start = static_cast<uint32_t>(startpos);
    d.prim_count = static_cast<uint32_t>(primcnt);
    d.base_vertex = basevert;
    uint32_t nstreams = 0;
    for (uint32_t i = 0; i < SG_MAX_STREAMS; ++i)
      if (streams_[i]) nstreams = i + 1;
    d.num_streams = nstreams;
    for (uint32_t i = 0; i < nstreams; ++i) {
      if (!streams_[i]) return result::failed;
      d.streams[i] = sg_vertex_stream{streams_[i]->handle(), static_cast<uint32_t>(strides_[i]),
                                      static_cast<uint32_t>(offsets_[i])};
    }
    d.num_inputs = static_cast<uint32_t>(layout_->registers.size());
    for (uint32_t i = 0; i < d.num_inputs; ++i) d.inputs[i] = layout_->registers[i];
    d.num_varyings = vs_code_ ? vs_code_->varyings : vs_->num_output_attributes();
    if (d.num_varyings > SG_MAX_VARYINGS) return result::invalid_parameter;
    for (uint32_t i = 0; i < d.num_varyings; ++i)
      d.varying_modifiers[i] = vs_code_ ? static_cast<uint32_t>(am::am_linear) : vs_->output_attribute_modifiers(i);
    raster_desc const& r = rs_->get_desc();
    d.raster = sg_raster_desc{static_cast<uint32_t>(r.fm), static_cast<uint32_t>(r.cm), r.front_ccw ? 1u : 0u, 0u};
    depth_stencil_desc const& s = dss_->get_desc();
    d.depth_stencil.depth_enable = s.depth_enable;
    d.depth_stencil.depth_write = s.depth_write_mask;
    d.depth_stencil.depth_func = s.depth_func;
    d.depth_stencil.stencil_enable = s.stencil_enable;
    d.depth_stencil.stencil_read_mask = s.stencil_read_mask;
    d.depth_stencil.stencil_write_mask = s.stencil_write_mask;
    d.depth_stencil.front = sg_stencil_face_desc{static_cast<uint32_t>(s.front_face.stencil_fail_op),
                                                 static_cast<uint32_t>(s.front_face.stencil_depth_fail_op),
                                                 static_cast<uint32_t>(s.front_face.stencil_pass_op),
                                                 static_cast<uint32_t>(s.front_face.stencil_func)};
    d.depth_stencil.back = sg_stencil_face_desc{static_cast<uint32_t>(s.back_face.stencil_fail_op),
                                                static_cast<uint32_t>(s.back_face.stencil_depth_fail_op),
                                                static_cast<uint32_t>(s.back_face.stencil_pass_op),
                                                static_cast<uint32_t>(s.back_face.stencil_func)};
    d.stencil_ref = stencil_ref_;
    result const rv = vs_code_ ? pack_code(*vs_code_, vs_vars_, vs_samplers_, d.vs) : vs_->pack(d.vs);
    result const rp = ps_code_ ? pack_code(*ps_code_, ps_vars_, ps_samplers_, d.ps) : ps_->pack(d.ps);
    if (rv != result::ok || rp != result::ok || bs_->pack(d.bs) != result::ok) return result::invalid_parameter;
    return result::ok;
  }

  // A compiled shader's program, its uniforms' words from the variables set
  // by name (missing ones are 0), its sampler, and a pixel shader's input
  // links to the compiled vertex shader's outputs (its own order with a cpp
  // vertex shader).
  result pack_code(shader::shader_object const& o, std::unordered_map<std::string, std::vector<uint8_t>> const& vars,
                   std::unordered_map<std::string, sampler_ptr> const& samps, sg_shader& s) const {
    std::memset(&s, 0, sizeof(s));
    if (sg_shader_register(dev_->dev, o.module, &s.program) != SG_OK) return result::failed;
    for (auto const& u : o.uniforms) {
      auto it = vars.find(u.name);
      if (it != vars.end())
        std::memcpy(&s.constants[u.word], it->second.data(), std::min<size_t>(it->second.size(), 4u * u.words));
    }
    if (!o.samplers.empty()) {
      auto it = samps.find(o.samplers[0]);
      s.samplers[0] = it != samps.end() && it->second ? it->second->handle() : 0;
    }
    if (o.language == shader::lang_pixel_shader && vs_code_) {
      uint32_t link = 0;
      for (auto const& in : o.inputs) {
        if (in.reg < 0) continue;
        for (auto const& out : vs_code_->outputs)
          if (out.reg >= 0 && salvia::detail::same_semantic(out.semantic, in.semantic) && out.index == in.index)
            link |= static_cast<uint32_t>(out.reg + 1) << (3 * in.reg);
      }
      std::memcpy(&s.constants[47], &link, sizeof link);
    }
    return result::ok;
  }

private:
  result submit(bool indexed, size_t startpos, size_t primcnt, int basevert) {
    sg_draw_desc d;
    result r = build_desc(indexed, startpos, primcnt, basevert, d);
    if (r != result::ok) return r;
    std::vector<std::shared_ptr<detail::query_counters>> qs;
    for (auto const& q : queries_) qs.push_back(q->counters);
    dev_->queue_draw(d, qs);
    return result::ok;
  }

  detail::device_sp dev_;
  buffer_ptr streams_[SG_MAX_STREAMS];
  size_t strides_[SG_MAX_STREAMS] = {}, offsets_[SG_MAX_STREAMS] = {};
  buffer_ptr ib_;
  format ib_fmt_ = format_r16_uint;  // renderer_impl's default (renderer_impl.cpp:269-284)
  primitive_topology topo_ = primitive_triangle_list;
  input_layout_ptr layout_;
  cpp_vertex_shader_ptr vs_;
  cpp_pixel_shader_ptr ps_;
  cpp_blend_shader_ptr bs_;
  shader::shader_object_ptr vs_code_, ps_code_;
  raster_state_ptr rs_;
  depth_stencil_state_ptr dss_;
  int32_t stencil_ref_ = 0;
  std::vector<surface_ptr> colors_;
  surface_ptr ds_;
  viewport vp_;
  std::vector<async_object_ptr> queries_;
  buffer_ptr mapped_buf_;
  surface_ptr mapped_surf_;
  map_mode mapped_mode_ = map_mode_none;
  std::vector<uint8_t> shadow_;
  std::unordered_map<std::string, std::vector<uint8_t>> vs_vars_, ps_vars_;
  std::unordered_map<std::string, sampler_ptr> vs_samplers_, ps_samplers_;

  static result keep(std::unordered_map<std::string, std::vector<uint8_t>>& vars, std::string const& name,
                     void const* data, size_t sz) {
    if (!data && sz) return result::invalid_parameter;
    auto const* b = static_cast<uint8_t const*>(data);
    vars[name].assign(b, b + sz);
    return result::ok;
  }
};
using renderer_ptr = std::shared_ptr<renderer>;

// Factories (renderer.h:133-134).  Both create a renderer on CUDA device 0 with
// a stream of its own; commands are stream-ordered, flush() waits for them.
inline renderer_ptr create_gpu_renderer(int cuda_device = 0, void* cuda_stream = nullptr) {
  sg_device* d = nullptr;
  if (sg_device_create(cuda_device, cuda_stream, &d) != SG_OK) return nullptr;
  return std::make_shared<renderer>(d);
}
inline renderer_ptr create_benchmark_renderer() { return create_gpu_renderer(0); }

// compile(code, lang) (renderer.h:136-147): null when the source does not
// translate (the translator's message goes to stderr) or the module does not
// build.
inline shader::shader_object_ptr compile(std::string const& code, shader::languages lang) {
  using translate_fn = int32_t (*)(char const*, uint32_t, char const*, char const*, char**, char**, char**);
  using free_fn = void (*)(char*);
  auto fail = [](std::string const& why) {
    std::fprintf(stderr, "compile: %s\n", why.c_str());
    return shader::shader_object_ptr();
  };
  void* lib = salvia::detail::sasl_library();
  if (!lib) return fail("the SASL translator (libsalvia_gb300.so) is not loaded");
  auto tr = reinterpret_cast<translate_fn>(dlsym(lib, "sg_sasl_translate"));
  auto fr = reinterpret_cast<free_fn>(dlsym(lib, "sg_sasl_free"));
  if (!tr || !fr) return fail("the library exports no SASL translator");
  bool const host_only = std::getenv("SALVIA_GB300_SASL_HOST_ONLY") != nullptr;
  char hex[24];
  std::snprintf(hex, sizeof hex, "%016zx", std::hash<std::string>{}(code + static_cast<char>('0' + lang)));
  auto obj = std::make_shared<shader::shader_object>();
  obj->language = lang;
  obj->cls = std::string("sasl_") + hex;
  char *src = nullptr, *refl = nullptr, *log = nullptr;
  int32_t const st = tr(code.c_str(), static_cast<uint32_t>(lang), nullptr, obj->cls.c_str(), &src, &refl, &log);
  if (st != SG_OK) {
    std::string const why = log ? std::string(log) : "status " + std::to_string(st);
    fr(log);
    return fail("the source does not translate: " + why);
  }
  obj->source = src;
  std::string const text = refl;
  fr(src);
  fr(refl);
  size_t at = 0;
  while (at < text.size()) {
    size_t const e = text.find('\n', at);
    std::string const line = text.substr(at, e == std::string::npos ? std::string::npos : e - at);
    at = e == std::string::npos ? text.size() : e + 1;
    char kind[16] = {0}, name[128] = {0};
    int a = 0, b = 0, c = 0;
    if (std::sscanf(line.c_str(), "%15s %127s %d %d %d", kind, name, &a, &b, &c) < 2) continue;
    std::string const k = kind;
    if (k == "input" || k == "output")
      (k == "input" ? obj->inputs : obj->outputs)
          .push_back({name, static_cast<uint32_t>(a), static_cast<int32_t>(b), static_cast<uint32_t>(c)});
    else if (k == "uniform")
      obj->uniforms.push_back({name, static_cast<uint32_t>(a), static_cast<uint32_t>(b)});
    else if (k == "sampler")
      obj->samplers.push_back(name);
    else if (k == "varyings")
      obj->varyings = static_cast<uint32_t>(std::atoi(name));
  }
  char const* cache = std::getenv("SALVIA_GB300_SHADER_CACHE");
  std::string const dir = cache ? cache : "/tmp/salvia_gb300_shaders";
  ::mkdir(dir.c_str(), 0755);
  std::string const so = dir + "/lib" + obj->cls + (host_only ? "_host" : "") + ".so";
  if (::access(so.c_str(), R_OK) != 0) {
    std::string const cu = dir + "/" + obj->cls + ".cu", tmp = so + "." + std::to_string(::getpid()) + ".tmp";
    std::ofstream(cu) << obj->source;
    std::string const root = salvia::detail::gb300_root(), inc = " -I" + root + "/include -I" + root + "/salviarenderer_gb300/csrc ";
    char const* nvcc = std::getenv("NVCC");
    if (!nvcc && ::access("/usr/local/cuda/bin/nvcc", X_OK) == 0) nvcc = "/usr/local/cuda/bin/nvcc";
    std::string const cmd =
        host_only ? std::string("g++ -std=c++17 -O2 -ffp-contract=off -fPIC -shared -x c++ ") + cu + inc + "-o " + tmp
                  : std::string(nvcc ? nvcc : "nvcc") +
                        " -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 -fmad=false -Xcompiler -ffp-contract=off"
                        " -shared -Xcompiler -fPIC -cudart shared " + cu + inc + "-o " + tmp;
    if (std::system(cmd.c_str()) != 0 || std::rename(tmp.c_str(), so.c_str()) != 0)
      return fail("building the shader module failed: " + cmd);
  }
  void* h = dlopen(so.c_str(), RTLD_NOW | RTLD_LOCAL);  // kept loaded: devices hold the module
  if (!h) return fail(std::string("loading the shader module failed: ") + dlerror());
  auto mod = reinterpret_cast<sg_shader_module const* (*)()>(dlsym(h, ("salvia_gb300_module_" + obj->cls).c_str()));
  if (!mod) return fail("the shader module exports no " + obj->cls);
  obj->module = mod();
  return obj;
}
inline shader::shader_object_ptr compile(std::string const& code, shader::shader_profile const& profile) {
  return compile(code, profile.language);
}
inline renderer_ptr create_software_renderer() { return create_gpu_renderer(0); }

}  // namespace salvia::core
